/*
 * ref_shim.h -- host stand-ins for the CUDA built-ins, intrinsics, inline-PTX
 * helpers (Util.hpp:72-151) and legacy texture/surface references that the
 * reference's device code uses, so that its .inl / .cu sources compile for
 * the host. Shared by the translation units of the reference harness.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref).
 */
#pragma once

#include <cuda.h>
#include <vector_types.h>
#include <vector_functions.h>

#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <ctime>

#pragma STDC FENV_ACCESS ON

// ---------------------------------------------------------------- CUDA shims
#define __device__
#define __host__
#define __inline__ inline
#define __forceinline__ inline
#define __shared__ static
#define __constant__
#define __global__
#define __launch_bounds__(a, b)

inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }
inline long long min(long long a, long long b) { return a < b ? a : b; }
inline long long max(long long a, long long b) { return a > b ? a : b; }
inline unsigned long long min(unsigned long long a, unsigned long long b) { return a < b ? a : b; }
inline unsigned long long max(unsigned long long a, unsigned long long b) { return a > b ? a : b; }
// CUDA's mixed signed/unsigned overloads compare as unsigned.
inline unsigned int min(unsigned int a, int b) { return min(a, (unsigned int)b); }
inline unsigned int min(int a, unsigned int b) { return min((unsigned int)a, b); }
inline unsigned int max(unsigned int a, int b) { return max(a, (unsigned int)b); }
inline unsigned int max(int a, unsigned int b) { return max((unsigned int)a, b); }

inline uint3 threadIdx, blockIdx;
inline dim3 blockDim, gridDim;

inline int __float_as_int(float f) { int i; std::memcpy(&i, &f, 4); return i; }
inline float __int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
inline double __longlong_as_double(long long v) { double d; std::memcpy(&d, &v, 8); return d; }
inline long long __double_as_longlong(double d) { long long v; std::memcpy(&v, &d, 8); return v; }
inline int __double2loint(double d) { return (int)(unsigned int)(unsigned long long)__double_as_longlong(d); }
inline int __double2hiint(double d) { return (int)(unsigned int)((unsigned long long)__double_as_longlong(d) >> 32); }
inline double __hiloint2double(int hi, int lo) {
    return __longlong_as_double((long long)(((unsigned long long)(unsigned int)hi << 32) | (unsigned int)lo));
}
inline int __popc(unsigned int v) { return __builtin_popcount(v); }
inline int __popcll(unsigned long long v) { return __builtin_popcountll(v); }
inline int __ffs(int v) { return __builtin_ffs(v); }
inline void __syncthreads() {}
inline unsigned int __ballot(int p) { return p ? (1u << (threadIdx.x & 31)) : 0u; }
inline int __any(int p) { return p; }
inline int __all(int p) { return p; }
inline int atomicAdd(int* p, int v) { int o = *p; *p += v; return o; }
inline unsigned int atomicAdd(unsigned int* p, unsigned int v) { unsigned int o = *p; *p += v; return o; }
inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) { unsigned long long o = *p; *p += v; return o; }
inline unsigned int atomicOr(unsigned int* p, unsigned int v) { unsigned int o = *p; *p |= v; return o; }

template <class T, int D> struct texture { const T* ptr; };
template <class T, int D> struct surface { unsigned char* ptr; long long pitch; };
template <class T> inline T tex1Dfetch(const texture<T, 1>& t, int i) { return t.ptr[i]; }
template <class T> inline T surf2Dread(const surface<void, 2>& s, int x, int y) {
    T v; std::memcpy(&v, s.ptr + (long long)y * s.pitch + x, sizeof(T)); return v;
}
template <class T> inline void surf2Dwrite(T v, const surface<void, 2>& s, int x, int y) {
    std::memcpy(s.ptr + (long long)y * s.pitch + x, &v, sizeof(T));
}

// The reference's Defs.hpp / Math.hpp (host flavour, FW_CUDA == 0).
#include "base/Math.hpp"
#include "cudaraster/cuda/Constants.hpp"

namespace FW {
// ------------------------------------------- Util.hpp:72-151 PTX helpers
static U32 g_carry = 0;
static int laneIdx() { return (int)(threadIdx.x & 31); }

inline U32 getLo(U64 a) { return (U32)a; }
inline S32 getLo(S64 a) { return (S32)(U32)(U64)a; }
inline U32 getHi(U64 a) { return (U32)(a >> 32); }
inline S32 getHi(S64 a) { return (S32)(U32)((U64)a >> 32); }
inline U64 combineLoHi(U32 lo, U32 hi) { return ((U64)hi << 32) | lo; }
inline S64 combineLoHi(S32 lo, S32 hi) { return (S64)(((U64)(U32)hi << 32) | (U32)lo); }
inline U32 getLaneMaskLt() { return (1u << laneIdx()) - 1u; }
inline U32 getLaneMaskLe() { return (U32)(((U64)2 << laneIdx()) - 1u); }
inline U32 getLaneMaskGt() { return ~getLaneMaskLe(); }
inline U32 getLaneMaskGe() { return ~getLaneMaskLt(); }
inline int findLeadingOne(U32 v) { return v ? 31 - __builtin_clz(v) : -1; }      // bfind.u32
inline bool singleLane() { return true; }
inline U32 add_cc(U32 a, U32 b) { U64 s = (U64)a + b; g_carry = (U32)(s >> 32); return (U32)s; }
inline U32 addc(U32 a, U32 b) { return a + b + g_carry; }
inline U32 addc_cc(U32 a, U32 b) { U64 s = (U64)a + b + g_carry; g_carry = (U32)(s >> 32); return (U32)s; }
inline S32 f32_to_s32_sat(F32 a) {        // cvt.rni.sat.s32.f32
    if (std::isnan(a)) return 0;
    if (a >= 2147483648.0f) return 0x7FFFFFFF;
    if (a <= -2147483648.0f) return (S32)0x80000000u;
    return (S32)std::nearbyint(a);
}
inline U32 f32_to_u32_sat(F32 a) {        // cvt.rni.sat.u32.f32
    if (!(a > 0.0f)) return 0;
    if (a >= 4294967296.0f) return 0xFFFFFFFFu;
    return (U32)std::nearbyint(a);
}
inline U32 f32_to_u32_sat_rmi(F32 a) {    // cvt.rmi.sat.u32.f32
    if (!(a >= 1.0f)) return 0;
    if (a >= 4294967296.0f) return 0xFFFFFFFFu;
    return (U32)std::floor(a);
}
inline U32 f32_to_u8_sat(F32 a) {         // cvt.rni.sat.u8.f32
    if (!(a > 0.0f)) return 0;
    if (a >= 255.0f) return 255;
    return (U32)std::nearbyint(a);
}
inline S64 f32_to_s64(F32 a) {            // cvt.rni.s64.f32
    if (std::isnan(a)) return 0;
    if (a >= 9223372036854775808.0f) return (S64)0x7FFFFFFFFFFFFFFFull;
    if (a <= -9223372036854775808.0f) return (S64)0x8000000000000000ull;
    return (S64)std::nearbyint(a);
}
inline S32 sh0(U32 v) { return (S32)(S16)(U16)(v & 0xFFFF); }
inline S32 sh1(U32 v) { return (S32)(S16)(U16)(v >> 16); }
inline S32 uh0(U32 v) { return (S32)(v & 0xFFFF); }
inline S32 uh1(U32 v) { return (S32)(v >> 16); }
inline U32 ub(U32 v, int i) { return (v >> (8 * i)) & 0xFF; }
inline S32 add_s16lo_s16lo(S32 a, S32 b) { return sh0(a) + sh0(b); }
inline S32 add_s16hi_s16lo(S32 a, S32 b) { return sh1(a) + sh0(b); }
inline S32 add_s16lo_s16hi(S32 a, S32 b) { return sh0(a) + sh1(b); }
inline S32 add_s16hi_s16hi(S32 a, S32 b) { return sh1(a) + sh1(b); }
inline S32 sub_s16lo_s16lo(S32 a, S32 b) { return sh0(a) - sh0(b); }
inline S32 sub_s16hi_s16lo(S32 a, S32 b) { return sh1(a) - sh0(b); }
inline S32 sub_s16lo_s16hi(S32 a, S32 b) { return sh0(a) - sh1(b); }
inline S32 sub_s16hi_s16hi(S32 a, S32 b) { return sh1(a) - sh1(b); }
inline S32 sub_u16lo_u16lo(U32 a, U32 b) { return uh0(a) - uh0(b); }
inline S32 sub_u16hi_u16lo(U32 a, U32 b) { return uh1(a) - uh0(b); }
inline S32 sub_u16lo_u16hi(U32 a, U32 b) { return uh0(a) - uh1(b); }
inline S32 sub_u16hi_u16hi(U32 a, U32 b) { return uh1(a) - uh1(b); }
inline U32 add_b0(U32 a, U32 b) { return ub(a, 0) + b; }
inline U32 add_b1(U32 a, U32 b) { return ub(a, 1) + b; }
inline U32 add_b2(U32 a, U32 b) { return ub(a, 2) + b; }
inline U32 add_b3(U32 a, U32 b) { return ub(a, 3) + b; }
inline U32 vmad_b0(U32 a, U32 b, U32 c) { return ub(a, 0) * b + c; }
inline U32 vmad_b1(U32 a, U32 b, U32 c) { return ub(a, 1) * b + c; }
inline U32 vmad_b2(U32 a, U32 b, U32 c) { return ub(a, 2) * b + c; }
inline U32 vmad_b3(U32 a, U32 b, U32 c) { return ub(a, 3) * b + c; }
inline U32 vmad_b0_b3(U32 a, U32 b, U32 c) { return ub(a, 0) * ub(b, 3) + c; }
inline U32 vmad_b1_b3(U32 a, U32 b, U32 c) { return ub(a, 1) * ub(b, 3) + c; }
inline U32 vmad_b2_b3(U32 a, U32 b, U32 c) { return ub(a, 2) * ub(b, 3) + c; }
inline U32 vmad_b3_b3(U32 a, U32 b, U32 c) { return ub(a, 3) * ub(b, 3) + c; }
inline U32 add_mask8(U32 a, U32 b) { return (a + b) & 0xFF; }
inline U32 sub_mask8(U32 a, U32 b) { return (a - b) & 0xFF; }
inline S32 max_max(S32 a, S32 b, S32 c) { return ::max(::max(a, b), c); }
inline S32 min_min(S32 a, S32 b, S32 c) { return ::min(::min(a, b), c); }
inline S32 max_add(S32 a, S32 b, S32 c) { return ::max(a, b) + c; }
inline S32 min_add(S32 a, S32 b, S32 c) { return ::min(a, b) + c; }
inline U32 add_add(U32 a, U32 b, U32 c) { return a + b + c; }
inline U32 sub_add(U32 a, U32 b, U32 c) { return a - b + c; }
inline U32 add_sub(U32 a, U32 b, U32 c) { return a - c + b; }
inline S32 add_clamp_0_x(S32 a, S32 b, S32 c) {  // vadd.u32.s32.s32.sat.min
    long long s = (long long)a + b;
    U32 t = s < 0 ? 0u : (s > 0xFFFFFFFFll ? 0xFFFFFFFFu : (U32)s);
    return (S32)::min(t, (U32)c);
}
inline S32 add_clamp_b0(S32 a, S32 b, S32 c) { long long s = (long long)a + b; U32 t = s < 0 ? 0 : (s > 255 ? 255 : (U32)s); return (S32)(((U32)c & ~0xFFu) | t); }
inline S32 add_clamp_b2(S32 a, S32 b, S32 c) { long long s = (long long)a + b; U32 t = s < 0 ? 0 : (s > 255 ? 255 : (U32)s); return (S32)(((U32)c & ~0xFF0000u) | (t << 16)); }
inline U32 prmt(U32 a, U32 b, U32 c) {
    U64 src = ((U64)b << 32) | a;
    U32 r = 0;
    for (int i = 0; i < 4; i++) {
        U32 sel = (c >> (4 * i)) & 0xF;
        U32 byte = (U32)(src >> (8 * (sel & 7))) & 0xFF;
        if (sel & 8) byte = (byte & 0x80) ? 0xFF : 0x00;
        r |= byte << (8 * i);
    }
    return r;
}
inline S32 u32lo_sext(U32 a) { return (S32)(S16)(U16)(a & 0xFFFF); }
inline U32 slct(U32 a, U32 b, S32 c) { return c >= 0 ? a : b; }
inline S32 slct(S32 a, S32 b, S32 c) { return c >= 0 ? a : b; }
inline F32 slct(F32 a, F32 b, S32 c) { return c >= 0 ? a : b; }
inline U32 isetge(S32 a, S32 b) { return a >= b ? 0xFFFFFFFFu : 0u; }
inline F64 rcp_approx(F64 a) { return 1.0 / a; }
inline F32 fma_rm(F32 a, F32 b, F32 c) {           // fma.rm.f32
    int old = std::fegetround();
    std::fesetround(FE_DOWNWARD);
    volatile F32 va = a, vb = b, vc = c;
    F32 r = std::fmaf(va, vb, vc);
    std::fesetround(old);
    return r;
}
template <class T> inline T cachedLoad(const T* p) { return *p; }
template <class T> inline void cachedStore(T* p, T v) { *p = v; }
template <class T> inline T uncachedLoad(const T* p) { return *p; }
template <class T> inline void uncachedStore(T* p, T v) { *p = v; }

// Util.hpp:153-176 declarations (the reference declares these only for nvcc).
U32 idiv_fast(U32 a, U32 b);
U32 toABGR(float4 color);
U32 blendABGR(U32 src, U32 dst, U32 srcColorFactor, U32 dstColorFactor, U32 srcAlphaFactor, U32 dstAlphaFactor);
U32 blendABGRClamp(U32 src, U32 dst, U32 srcColorFactor, U32 dstColorFactor, U32 srcAlphaFactor, U32 dstAlphaFactor);
uint3 setupPleq(float3 values, int2 v0, int2 d1, int2 d2, F32 areaRcp, int samplesLog2);
U64 cover8x8_exact_ref(S32 ox, S32 oy, S32 dx, S32 dy);
U64 cover8x8_conservative_ref(S32 ox, S32 oy, S32 dx, S32 dy);
U64 cover8x8_generateMask_ref(S64 curr, S64 stepX, S64 stepY);
bool cover8x8_missesTile(S32 ox, S32 oy, S32 dx, S32 dy);
void cover8x8_setupLUT(volatile U64* lut);
U64 cover8x8_exact_fast(S32 ox, S32 oy, S32 dx, S32 dy, U32 flips, volatile const U64* lut);
U64 cover8x8_conservative_fast(S32 ox, S32 oy, S32 dx, S32 dy, U32 flips, volatile const U64* lut);
U64 cover8x8_lookupMask(S64 yinit, U32 yinc, U32 flips, volatile const U64* lut);
U64 cover8x8_exact_noLUT(S32 ox, S32 oy, S32 dx, S32 dy);
U64 cover8x8_conservative_noLUT(S32 ox, S32 oy, S32 dx, S32 dy);
U64 cover8x8_generateMask_noLUT(S32 curr, S32 dx, S32 dy);
U32 coverMSAA_ref(int samplesLog2, S32 ox, S32 oy, S32 dx, S32 dy);
U32 coverMSAA_fast(int samplesLog2, S32 ox, S32 oy, S32 dx, S32 dy);
template <class T> void sortShared(T* ptr, int numItems);
}  // namespace FW

