// ShaderMath.hpp -- exactly specified arithmetic for shaders.
//
// The reference's example shaders (test/shader/Shaders.cu) call powf, log2f,
// normalize (a reciprocal square root) and tex2D on a bilinear texture. Under
// nvcc those are library or texture-unit approximations whose results are not
// specified, so no CPU oracle can reproduce them bit for bit. The functions
// here replace them with operations that are each correctly rounded
// (__fadd_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn, floorf), so a shader built on
// them is a pure function of its inputs that a CPU restatement matches
// exactly:
//
//   crLog2     log2 by the atanh series log2(m) = (2 / ln 2) * sum over k of
//              t^(2k+1) / (2k+1), t = (m - 1) / (m + 1), for the mantissa m
//              folded into [sqrt(1/2), sqrt(2)];
//   crExp2     2^z = 2^n * sqrt(2) * 2^f, f = z - n - 1/2 in [-1/2, 1/2), with
//              2^f by its Taylor series sum (f ln 2)^k / k!;
//   crPow      x^y = crExp2(y * crLog2(x)), within about 1e-5 relative of the
//              true power for the arguments lighting uses;
//   crNormalize  v * (1 * (1 / sqrt(dot(v, v)))), a zero vector staying zero,
//              as the reference framework writes normalized() (Math.hpp:112-202);
//   crTex2D    bilinear filtering of an RGBA8 atlas with normalized, wrapped
//              coordinates and 8-bit fractional weights -- the texture unit's
//              documented filter (x' = frac(u) * W - 1/2, i = floor(x'),
//              alpha = frac(x') in fixed point with 8 fractional bits), here
//              with the weight rounded to nearest and the weighted sum formed
//              in integers, then divided by 255 * 65536 once.
#pragma once

#include <cuda_runtime.h>

#include "Types.hpp"

namespace FW {

__device__ __forceinline__ F32 crPow2i(int e) { return __uint_as_float((U32)(e + 127) << 23); }  // e in [-126, 127]

// log2(x) for finite x > 0.
__device__ __forceinline__ F32 crLog2Finite(F32 x) {
    U32 b = __float_as_uint(x);
    S32 k = 0;
    if ((b >> 23) == 0u) {  // subnormal: scale by 2^24 first
        x = __fmul_rn(x, 16777216.0f);
        b = __float_as_uint(x);
        k = -24;
    }
    k += (S32)(b >> 23) - 127;
    F32 m = __uint_as_float((b & 0x7FFFFFu) | 0x3F800000u);  // [1, 2)
    if (m > 1.41421354f) {
        m = __fmul_rn(m, 0.5f);
        k += 1;
    }
    const F32 t = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const F32 t2 = __fmul_rn(t, t);
    F32 p = 0.26230818f;  // (2 / ln 2) / 11
    p = __fadd_rn(__fmul_rn(p, t2), 0.3205989f);   // / 9
    p = __fadd_rn(__fmul_rn(p, t2), 0.41219857f);  // / 7
    p = __fadd_rn(__fmul_rn(p, t2), 0.57707804f);  // / 5
    p = __fadd_rn(__fmul_rn(p, t2), 0.9617967f);   // / 3
    p = __fadd_rn(__fmul_rn(p, t2), 2.88539f);     // / 1
    return __fadd_rn((F32)k, __fmul_rn(t, p));
}

// log2 over the whole domain: 0 -> -inf, negative -> NaN, inf -> inf, NaN -> NaN.
__device__ __forceinline__ F32 crLog2(F32 x) {
    if (x != x) return x;
    if (x == 0.0f) return __uint_as_float(0xFF800000u);
    if (x < 0.0f) return __uint_as_float(0x7FC00000u);
    if (x == __uint_as_float(0x7F800000u)) return x;
    return crLog2Finite(x);
}

__device__ __forceinline__ F32 crExp2(F32 z) {
    if (z != z) return z;
    if (z >= 128.0f) return __uint_as_float(0x7F800000u);
    if (!(z > -150.0f)) return 0.0f;
    const F32 n = floorf(z);
    const F32 f = __fsub_rn(__fsub_rn(z, n), 0.5f);  // [-1/2, 1/2)
    F32 p = 1.0178086e-07f;                          // (ln 2)^9 / 9!
    p = __fadd_rn(__fmul_rn(p, f), 1.3215487e-06f);  // (ln 2)^8 / 8!
    p = __fadd_rn(__fmul_rn(p, f), 1.5252734e-05f);
    p = __fadd_rn(__fmul_rn(p, f), 1.540353e-04f);
    p = __fadd_rn(__fmul_rn(p, f), 1.3333558e-03f);
    p = __fadd_rn(__fmul_rn(p, f), 9.618129e-03f);
    p = __fadd_rn(__fmul_rn(p, f), 5.550411e-02f);
    p = __fadd_rn(__fmul_rn(p, f), 2.402265e-01f);
    p = __fadd_rn(__fmul_rn(p, f), 6.931472e-01f);   // ln 2
    p = __fadd_rn(__fmul_rn(p, f), 1.0f);
    p = __fmul_rn(p, 1.4142135f);                    // sqrt(2)
    S32 ni = (S32)n;
    if (ni < -126) {
        p = __fmul_rn(p, crPow2i(-64));
        ni += 64;
    }
    return __fmul_rn(p, crPow2i(ni));
}

// x^y for x >= 0 (lighting's powf(max(-dot(I, R), 0), glossiness)).
__device__ __forceinline__ F32 crPow(F32 x, F32 y) {
    if (y == 0.0f) return 1.0f;
    if (!(x > 0.0f)) return y > 0.0f ? 0.0f : __uint_as_float(0x7F800000u);
    if (x == __uint_as_float(0x7F800000u)) return y > 0.0f ? x : 0.0f;
    return crExp2(__fmul_rn(y, crLog2Finite(x)));
}

// dot(a, b) summed left to right from zero (Math.hpp: VectorBase::dot).
__device__ __forceinline__ F32 crDot(const Vec3f& a, const Vec3f& b) {
    return __fadd_rn(__fadd_rn(__fadd_rn(0.0f, __fmul_rn(a.x, b.x)), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

__device__ __forceinline__ Vec3f crNormalize(const Vec3f& v) {
    const F32 len = __fsqrt_rn(crDot(v, v));
    const F32 s = __fmul_rn(1.0f, len != 0.0f ? __frcp_rn(len) : 0.0f);  // 1 / len, correctly rounded
    return Vec3f(__fmul_rn(v.x, s), __fmul_rn(v.y, s), __fmul_rn(v.z, s));
}

// evaluateLighting (test/shader/Shaders.cu:37-50): diffuse 0.25 + 0.75 *
// max(-dot(I, N), 0), specular max(-dot(I, R), 0)^glossiness with R the
// reflection of the view ray I about N.
__device__ __forceinline__ Vec3f evaluateLighting(const Vec3f& cameraPos, const Vec3f& cameraNormal,
                                                  const Vec3f& specularColor, F32 glossiness,
                                                  const Vec3f& diffuseColor) {
    const Vec3f I = crNormalize(cameraPos);
    const Vec3f N = crNormalize(cameraNormal);
    const F32 dotIN = crDot(I, N);
    const F32 twice = __fmul_rn(dotIN, 2.0f);
    const Vec3f R(__fsub_rn(I.x, __fmul_rn(N.x, twice)), __fsub_rn(I.y, __fmul_rn(N.y, twice)),
                  __fsub_rn(I.z, __fmul_rn(N.z, twice)));
    const F32 diffuseCoef = __fadd_rn(__fmul_rn(fmaxf(-dotIN, 0.0f), 0.75f), 0.25f);
    const F32 specularCoef = crPow(fmaxf(-crDot(I, R), 0.0f), glossiness);
    return Vec3f(__fadd_rn(__fmul_rn(diffuseCoef, diffuseColor.x), __fmul_rn(specularCoef, specularColor.x)),
                 __fadd_rn(__fmul_rn(diffuseCoef, diffuseColor.y), __fmul_rn(specularCoef, specularColor.y)),
                 __fadd_rn(__fmul_rn(diffuseCoef, diffuseColor.z), __fmul_rn(specularCoef, specularColor.z)));
}

// An RGBA8 texture atlas in device memory: one word per texel, R in the low
// byte (the surface word layout), rows of `width` words.
struct TextureAtlas {
    const U32* texels;
    S32 width, height;
};

// One axis of the filter: the two wrapped texel indices and the weight of the
// second, in 1/256 (0..256).
__device__ __forceinline__ void crTexAxis(F32 u, S32 n, S32& i0, S32& i1, U32& w) {
    F32 f = __fsub_rn(u, floorf(u));
    if (!(f >= 0.0f && f < 1.0f)) f = 0.0f;  // NaN or inf, or a wrap that rounded up to 1
    const F32 x = __fsub_rn(__fmul_rn(f, (F32)n), 0.5f);
    const F32 fl = floorf(x);
    const S32 i = (S32)fl;  // -1 .. n
    w = (U32)__float2int_rn(__fmul_rn(__fsub_rn(x, fl), 256.0f));
    i0 = i < 0 ? i + n : (i >= n ? i - n : i);
    i1 = i0 + 1 == n ? 0 : i0 + 1;
}

// s / (255 * 65536), correctly rounded, for integers 0 <= s <= 255 * 65536:
// RN(s / 255) by one multiplication by RN(1 / 255) and one FMA-based
// correction (Markstein), then the exact scaling by 2^-16. Equal to the IEEE
// division for every s in the range -- checked exhaustively on the CPU with
// IEEE fmaf -- at three instructions instead of a division.
__device__ __forceinline__ F32 crTexNormalize(U32 s) {
    const F32 x = (F32)s;  // < 2^24: exact
    const F32 rcp = 0.00392156886f;  // RN(1 / 255)
    const F32 q0 = __fmul_rn(x, rcp);
    const F32 r = __fmaf_rn(-q0, 255.0f, x);
    const F32 q = __fmaf_rn(r, rcp, q0);
    return __fmul_rn(q, 1.52587890625e-05f);  // 2^-16
}

// tex2D of an atlas with linear filtering, wrap addressing and normalized
// coordinates, returning channels in [0, 1].
__device__ __forceinline__ Vec4f crTex2D(const TextureAtlas& t, F32 u, F32 v) {
    S32 x0, x1, y0, y1;
    U32 a, b;
    crTexAxis(u, t.width, x0, x1, a);
    crTexAxis(v, t.height, y0, y1, b);
    const U32* r0 = t.texels + (S64)y0 * t.width;
    const U32* r1 = t.texels + (S64)y1 * t.width;
    const U32 c00 = __ldg(r0 + x0), c10 = __ldg(r0 + x1), c01 = __ldg(r1 + x0), c11 = __ldg(r1 + x1);
    const U32 w00 = (256u - a) * (256u - b), w10 = a * (256u - b), w01 = (256u - a) * b, w11 = a * b;
    F32 out[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int sh = 8 * k;
        const U32 s = w00 * ((c00 >> sh) & 255u) + w10 * ((c10 >> sh) & 255u) + w01 * ((c01 >> sh) & 255u) +
                      w11 * ((c11 >> sh) & 255u);  // < 2^24: exact as a float
        out[k] = crTexNormalize(s);  // s / (255 * 65536)
    }
    return Vec4f(out[0], out[1], out[2], out[3]);
}

}  // namespace FW
