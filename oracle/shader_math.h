/*
 * shader_math.h -- host restatement of the exactly specified shader
 * arithmetic of include/cudaraster/ShaderMath.hpp: log2 by the atanh series,
 * exp2 by the Taylor series of 2^f around f = 1/2, their power, the
 * framework's dot / normalize, evaluateLighting (test/shader/Shaders.cu:
 * 37-50) and the RGBA8 atlas filter that stands for the reference's tex2D.
 * Binary32, one correctly rounded operation at a time (compile with
 * -ffp-contract=off).
 *
 * TEST INFRASTRUCTURE ONLY: shared by the oracle and the reference harness.
 */
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace crsm {

typedef int32_t S32;
typedef uint32_t U32;
typedef int64_t S64;
typedef float F32;

// The reference's Shaders.cu calls log2f, powf, a reciprocal square root and
// tex2D, whose results nvcc does not specify; the pipeline replaces them with
// correctly rounded operations, restated here one operation at a time.
inline F32 pow2i(int e) { U32 b = (U32)(e + 127) << 23; F32 f; std::memcpy(&f, &b, 4); return f; }
inline U32 fbits(F32 f) { U32 b; std::memcpy(&b, &f, 4); return b; }
inline F32 bitsf(U32 b) { F32 f; std::memcpy(&f, &b, 4); return f; }

inline F32 log2_finite(F32 x) {  // finite x > 0: atanh series on the mantissa folded into [sqrt(1/2), sqrt(2)]
    U32 b = fbits(x);
    S32 k = 0;
    if ((b >> 23) == 0u) { x = x * 16777216.0f; b = fbits(x); k = -24; }
    k += (S32)(b >> 23) - 127;
    F32 m = bitsf((b & 0x7FFFFFu) | 0x3F800000u);
    if (m > 1.41421354f) { m = m * 0.5f; k += 1; }
    const F32 t = (m - 1.0f) / (m + 1.0f);
    const F32 t2 = t * t;
    F32 p = 0.26230818f;
    p = p * t2 + 0.3205989f;
    p = p * t2 + 0.41219857f;
    p = p * t2 + 0.57707804f;
    p = p * t2 + 0.9617967f;
    p = p * t2 + 2.88539f;
    return (F32)k + t * p;
}

inline F32 log2_full(F32 x) {
    if (x != x) return x;
    if (x == 0.0f) return -INFINITY;
    if (x < 0.0f) return NAN;
    if (std::isinf(x)) return x;
    return log2_finite(x);
}

inline F32 exp2_exact(F32 z) {  // 2^n * sqrt(2) * 2^f, 2^f by its Taylor series
    if (z != z) return z;
    if (z >= 128.0f) return INFINITY;
    if (!(z > -150.0f)) return 0.0f;
    const F32 n = std::floor(z);
    const F32 f = (z - n) - 0.5f;
    F32 p = 1.0178086e-07f;
    p = p * f + 1.3215487e-06f;
    p = p * f + 1.5252734e-05f;
    p = p * f + 1.540353e-04f;
    p = p * f + 1.3333558e-03f;
    p = p * f + 9.618129e-03f;
    p = p * f + 5.550411e-02f;
    p = p * f + 2.402265e-01f;
    p = p * f + 6.931472e-01f;
    p = p * f + 1.0f;
    p = p * 1.4142135f;
    S32 ni = (S32)n;
    if (ni < -126) { p = p * pow2i(-64); ni += 64; }
    return p * pow2i(ni);
}

inline F32 pow_exact(F32 x, F32 y) {
    if (y == 0.0f) return 1.0f;
    if (!(x > 0.0f)) return y > 0.0f ? 0.0f : INFINITY;
    if (std::isinf(x)) return y > 0.0f ? x : 0.0f;
    return exp2_exact(y * log2_finite(x));
}

inline F32 dot3(const F32 a[3], const F32 b[3]) { return ((0.0f + a[0] * b[0]) + a[1] * b[1]) + a[2] * b[2]; }

inline void normalize3(const F32 v[3], F32 r[3]) {  // v * (1 * rcp(length)), rcp(0) = 0
    const F32 len = std::sqrt(dot3(v, v));
    const F32 s = 1.0f * (len != 0.0f ? 1.0f / len : 0.0f);
    for (int k = 0; k < 3; k++) r[k] = v[k] * s;
}

// test/shader/Shaders.cu:37-50 evaluateLighting.
inline void evaluate_lighting(const F32 cameraPos[3], const F32 cameraNormal[3], const F32 spec[3], F32 gloss,
                       const F32 diffuse[3], F32 out[3]) {
    F32 I[3], N[3], R[3];
    normalize3(cameraPos, I);
    normalize3(cameraNormal, N);
    const F32 dotIN = dot3(I, N);
    const F32 twice = dotIN * 2.0f;
    for (int k = 0; k < 3; k++) R[k] = I[k] - N[k] * twice;
    const F32 diffuseCoef = std::fmax(-dotIN, 0.0f) * 0.75f + 0.25f;
    const F32 specularCoef = pow_exact(std::fmax(-dot3(I, R), 0.0f), gloss);
    for (int k = 0; k < 3; k++) out[k] = diffuseCoef * diffuse[k] + specularCoef * spec[k];
}

// Bilinear RGBA8 atlas lookup: wrap, normalized coordinates, 8-bit weights
// rounded to nearest, integer weighted sum / (255 * 65536).
inline void tex_axis(F32 u, S32 n, S32* i0, S32* i1, U32* w) {
    F32 f = u - std::floor(u);
    if (!(f >= 0.0f && f < 1.0f)) f = 0.0f;
    const F32 x = f * (F32)n - 0.5f;
    const F32 fl = std::floor(x);
    const S32 i = (S32)fl;
    *w = (U32)(S32)std::nearbyint((x - fl) * 256.0f);
    *i0 = i < 0 ? i + n : (i >= n ? i - n : i);
    *i1 = *i0 + 1 == n ? 0 : *i0 + 1;
}

inline void tex2d(const U32* atlas, S32 w, S32 h, F32 u, F32 v, F32 out[4]) {
    S32 x0, x1, y0, y1;
    U32 a, b;
    tex_axis(u, w, &x0, &x1, &a);
    tex_axis(v, h, &y0, &y1, &b);
    const U32 c00 = atlas[(S64)y0 * w + x0], c10 = atlas[(S64)y0 * w + x1];
    const U32 c01 = atlas[(S64)y1 * w + x0], c11 = atlas[(S64)y1 * w + x1];
    const U32 w00 = (256u - a) * (256u - b), w10 = a * (256u - b), w01 = (256u - a) * b, w11 = a * b;
    for (int k = 0; k < 4; k++) {
        const int sh = 8 * k;
        const U32 sum = w00 * ((c00 >> sh) & 255u) + w10 * ((c10 >> sh) & 255u) + w01 * ((c01 >> sh) & 255u) +
                        w11 * ((c11 >> sh) & 255u);
        out[k] = (F32)sum / 16711680.0f;
    }
}

}  // namespace crsm
