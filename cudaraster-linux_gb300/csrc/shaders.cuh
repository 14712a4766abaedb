// shaders.cuh -- fragment shaders of the built-in pipes (beyond the common
// ones in PixelPipe.hpp).
#pragma once

#include "cudaraster/PixelPipe.hpp"

namespace FW {

// Constant red, the reference's demo shader (test/shader/PassThrough.cu:44-54).
class FragmentShader_passthrough : public FragmentShaderBase {
public:
    __device__ __forceinline__ void run(void) { m_color = toABGR(Vec4f(Vec3f(1.0f, 0.0f, 0.0f), 1.0f)); }
};

// Colour from a hash of the triangle index: every triangle gets a distinct
// opaque colour, so any reordering of fragments shows up in the output.
class TriHashShader : public FragmentShaderBase {
public:
    __device__ __forceinline__ void run(void) {
        U32 h = (U32)m_triIdx * 2654435761u;
        h ^= h >> 15;
        h *= 2246822519u;
        h ^= h >> 13;
        m_color = h | 0xFF000000u;
    }
};

// Quad-mode probe: numerical derivatives of the barycentric u across the
// 2x2 quad drive the colour.
class DerivShader : public FragmentShaderBase {
public:
    __device__ __forceinline__ void run(void) {
        F32 u = m_center.y;
        F32 dx = dFdx(u), dy = dFdy(u);
        m_color = toABGR(Vec4f(__fmul_rn(fabsf(dx), 64.0f), __fmul_rn(fabsf(dy), 64.0f), m_center.z, 1.0f));
    }
};

template <> struct FragmentShaderTraits<FragmentShader_passthrough> { static constexpr bool mayDiscard = false; };
template <> struct FragmentShaderTraits<TriHashShader> { static constexpr bool mayDiscard = false; };
template <> struct FragmentShaderReads<FragmentShader_passthrough> {
    static constexpr bool center = false;
    static constexpr bool centroid = false;
};
template <> struct FragmentShaderReads<TriHashShader> {
    static constexpr bool center = false;
    static constexpr bool centroid = false;
};

}  // namespace FW
