// PixelPipe.hpp -- device-side public interface for pixel pipes.
//
// Same names and meaning as the reference's src/cudaraster/cuda/PixelPipe.hpp
// (render-mode flags :30-35, ShadedVertexBase :41-47, FragmentShaderBase
// :53-97, BlendShaderBase :103-124, the common shaders :130-175), so a pipe
// written for the reference compiles against this header:
//
//   #include <cudaraster/PixelPipe.inl>
//   CR_DEFINE_PIXEL_PIPE(MyPipe, MyVertex, MyFragmentShader, BlendSrcOver, 2,
//                        RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
//
// Differences: varyings are read with plain global loads instead of a
// texture reference, and the small vector types below are this project's
// own (FW::Vec2i/Vec3i/Vec2f/Vec3f/Vec4f with the operators shaders use).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "Types.hpp"

namespace FW {

// Component-wise arithmetic, each operation rounded on its own (no FMA
// contraction), as the reference source reads.
__device__ __forceinline__ Vec4f operator*(const Vec4f& a, F32 s) {
    return Vec4f(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s));
}
__device__ __forceinline__ Vec4f operator+(const Vec4f& a, const Vec4f& b) {
    return Vec4f(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
}
__device__ __forceinline__ Vec4f operator-(const Vec4f& a, const Vec4f& b) {
    return Vec4f(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __fsub_rn(a.w, b.w));
}
__device__ __forceinline__ Vec3f operator*(const Vec3f& a, F32 s) {
    return Vec3f(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s));
}
__device__ __forceinline__ Vec3f operator+(const Vec3f& a, const Vec3f& b) {
    return Vec3f(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
__device__ __forceinline__ Vec3f operator-(const Vec3f& a, const Vec3f& b) {
    return Vec3f(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}

// -------------------------------------------------- render mode flags (:30-35)
enum {
    RenderModeFlag_EnableDepth = 1 << 0,  // depth test LESS + depth write
    RenderModeFlag_EnableLerp = 1 << 1,   // perspective-correct varying interpolation
    RenderModeFlag_EnableQuads = 1 << 2,  // 2x2 quads, numerical derivatives
};

// -------------------------------------------------------------- base types
struct ShadedVertexBase {
    Vec4f clipPos;  // subclasses append one Vec4f per varying, nothing else
};

class FragmentShaderBase {
public:
    __device__ __forceinline__ Vec4f getVaryingAtVertex(int varyingIdx, int vertIdx) const {
        const float4* p = m_vertices + (S64)vertIdx * (m_vertexBytes >> 4) + varyingIdx + 1;
        float4 t = __ldg(p);
        return Vec4f(t.x, t.y, t.z, t.w);
    }
    // v0 * b.x + v1 * b.y + v2 * b.z (PixelPipe.inl:53-59)
    __device__ __forceinline__ Vec4f interpolateVarying(int varyingIdx, const Vec3f& bary) const {
        Vec4f v0 = getVaryingAtVertex(varyingIdx, m_vertIdx.x);
        Vec4f v1 = getVaryingAtVertex(varyingIdx, m_vertIdx.y);
        Vec4f v2 = getVaryingAtVertex(varyingIdx, m_vertIdx.z);
        return v0 * bary.x + v1 * bary.y + v2 * bary.z;
    }
    // Numerical derivatives across the 2x2 quad (quad mode only). All lanes
    // of the pass must call these together.
    __device__ __forceinline__ F32 dFdx(F32 v) const { return quadDiff(v, 1); }
    __device__ __forceinline__ F32 dFdy(F32 v) const { return quadDiff(v, 2); }
    __device__ __forceinline__ Vec2f dFdx(const Vec2f& v) const { return Vec2f(dFdx(v.x), dFdx(v.y)); }
    __device__ __forceinline__ Vec2f dFdy(const Vec2f& v) const { return Vec2f(dFdy(v.x), dFdy(v.y)); }
    __device__ __forceinline__ Vec3f dFdx(const Vec3f& v) const { return Vec3f(dFdx(v.x), dFdx(v.y), dFdx(v.z)); }
    __device__ __forceinline__ Vec3f dFdy(const Vec3f& v) const { return Vec3f(dFdy(v.x), dFdy(v.y), dFdy(v.z)); }
    __device__ __forceinline__ Vec4f dFdx(const Vec4f& v) const { return Vec4f(dFdx(v.x), dFdx(v.y), dFdx(v.z), dFdx(v.w)); }
    __device__ __forceinline__ Vec4f dFdy(const Vec4f& v) const { return Vec4f(dFdy(v.x), dFdy(v.y), dFdy(v.z), dFdy(v.w)); }

    __device__ __forceinline__ void run(void) {}

    // Inputs.
    S32 m_triIdx;             // triangle index within the draw
    Vec3i m_vertIdx;          // vertex indices
    Vec2i m_pixelPos;         // integer pixel position
    S32 m_vertexBytes;        // sizeof(vertex struct)
    volatile F32* m_shared;   // 32 entries for the warp
    Vec3f m_center;           // barycentrics at the pixel centre
    Vec3f m_centerDX;
    Vec3f m_centerDY;
    Vec3f m_centroid;         // barycentrics at the centroid of the covered samples
    Vec3f m_centroidDX;
    Vec3f m_centroidDY;
    // Outputs.
    U32 m_color;              // ABGR8
    bool m_discard;
    // Set by the pipeline.
    const float4* m_vertices;
    U32 m_laneMask;           // lanes of the warp running the shader together

private:
    __device__ __forceinline__ F32 quadDiff(F32 v, int bit) const {
        const int lane = threadIdx.x & 31;
        __syncwarp(m_laneMask);
        m_shared[lane] = v;
        __syncwarp(m_laneMask);
        F32 r = __fsub_rn(m_shared[lane | bit], m_shared[lane & ~bit]);
        __syncwarp(m_laneMask);
        return r;
    }
};

class BlendShaderBase {
public:
    __device__ __forceinline__ bool needsDst(void) { return true; }  // must be a constant
    __device__ __forceinline__ void run(void) {}
    S32 m_triIdx;
    Vec2i m_pixelPos;
    S32 m_sampleIdx;
    U32 m_src;
    U32 m_dst;
    U32 m_color;
    bool m_writeColor;
};

// toABGR (Util.inl:30-38): fma.rm + cvt.rmi.sat per channel, top byte.
__device__ __forceinline__ U32 toABGR(const Vec4f& c) {
    const F32 scale = (F32)(1 << 24) * 255.0f, bias = (F32)(1 << 24) * 0.5f;
    U32 x = __float2uint_rd(__fmaf_rd(c.x, scale, bias)) >> 24;
    U32 y = __float2uint_rd(__fmaf_rd(c.y, scale, bias)) >> 24;
    U32 z = __float2uint_rd(__fmaf_rd(c.z, scale, bias)) >> 24;
    U32 w = __float2uint_rd(__fmaf_rd(c.w, scale, bias)) >> 24;
    return x | (y << 8) | (z << 16) | (w << 24);
}

// blendABGR / blendABGRClamp (Util.inl:42-60). Factors use their top byte.
__device__ __forceinline__ U32 blendABGRImpl(U32 src, U32 dst, U32 scf, U32 dcf, U32 saf, U32 daf, bool clamp) {
    U32 out = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        U32 s = (src >> (8 * c)) & 0xFF, d = (dst >> (8 * c)) & 0xFF;
        U32 t = (c < 3) ? (s * (scf >> 24) + d * (dcf >> 24)) : (s * (saf >> 24) + d * (daf >> 24));
        if (clamp) t = t < 255u * 255u ? t : 255u * 255u;
        out |= ((t * 0x010101u + 0x800000u) >> 24) << (8 * c);
    }
    return out;
}
__device__ __forceinline__ U32 blendABGR(U32 src, U32 dst, U32 scf, U32 dcf, U32 saf, U32 daf) {
    return blendABGRImpl(src, dst, scf, dcf, saf, daf, false);
}
__device__ __forceinline__ U32 blendABGRClamp(U32 src, U32 dst, U32 scf, U32 dcf, U32 saf, U32 daf) {
    return blendABGRImpl(src, dst, scf, dcf, saf, daf, true);
}

// ----------------------------------------------------------- common shaders
struct GouraudVertex : ShadedVertexBase {
    Vec4f color;  // varying 0
};

class GouraudShader : public FragmentShaderBase {
public:
    __device__ __forceinline__ void run(void) { m_color = toABGR(interpolateVarying(0, m_centroid)); }
};

class BlendReplace : public BlendShaderBase {  // dst = src
public:
    __device__ __forceinline__ bool needsDst(void) { return false; }
    __device__ __forceinline__ void run(void) { m_color = m_src; }
};

class BlendSrcOver : public BlendShaderBase {  // dst = lerp(dst, src, src.a)
public:
    __device__ __forceinline__ void run(void) { m_color = blendABGR(m_src, m_dst, m_src, ~m_src, m_src, ~m_src); }
};

class BlendAdditive : public BlendShaderBase {  // dst += src
public:
    __device__ __forceinline__ void run(void) { m_color = blendABGRClamp(m_src, m_dst, ~0u, ~0u, ~0u, ~0u); }
};

class BlendDepthOnly : public BlendShaderBase {  // dst = dst
public:
    __device__ __forceinline__ bool needsDst(void) { return false; }
    __device__ __forceinline__ void run(void) { m_writeColor = false; }
};

// ---------------------------------------------------------- shader traits
// Compile-time facts the fine stage uses to pick its algorithm. With depth
// testing on, a blend shader that ignores the destination and a fragment
// shader that never discards, the colour and depth of every sample depend
// only on the front-most covering fragment (earliest in submission order on
// ties), so the fine stage resolves visibility first and shades each sample's
// winner once. A fragment shader that never discards also lets the ordered
// path (blending pipes) drop, at one sample per pixel, the fragments that
// would fail the depth test behind an earlier one of the same batch. The
// defaults are the safe ones; specialise them for your own shaders only when
// the facts hold (a shader that can discard must keep mayDiscard true).
template <class BS> struct BlendShaderTraits { static constexpr bool needsDst = true; };
template <> struct BlendShaderTraits<BlendReplace> { static constexpr bool needsDst = false; };
template <> struct BlendShaderTraits<BlendDepthOnly> { static constexpr bool needsDst = false; };
template <class FS> struct FragmentShaderTraits { static constexpr bool mayDiscard = true; };
template <> struct FragmentShaderTraits<GouraudShader> { static constexpr bool mayDiscard = false; };
// Which barycentrics a fragment shader reads: the pixel centre's
// (m_center, m_centerDX, m_centerDY) and the centroid's (m_centroid ...).
// The fine stage skips computing the ones a shader never reads; with one
// sample per pixel both are the same values.
template <class FS> struct FragmentShaderReads {
    static constexpr bool center = true;
    static constexpr bool centroid = true;
};
template <> struct FragmentShaderReads<GouraudShader> {
    static constexpr bool center = false;
    static constexpr bool centroid = true;
};

// Profiling modes (PixelPipe.hpp:208-213). Only the default mode (per-stage
// events + device counters) exists here.
#define ProfilingMode_Default 0
#define ProfilingMode_Counters 1
#define ProfilingMode_Timers 2

}  // namespace FW
