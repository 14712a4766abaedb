/*
 * cr_oracle.cpp -- scalar CPU restatement of the reference rasterizer.
 *
 * TEST INFRASTRUCTURE ONLY (see cr_oracle.h). Every function cites the
 * reference file:line it restates (paths relative to
 * tcoppex/cudaraster-linux/src/cudaraster/). Compile with
 * -ffp-contract=off: the normative arithmetic is binary32 evaluated one
 * operation at a time, exactly as the reference source is written.
 *
 * The fine stage is restated in its sequential meaning: for every tile, the
 * subtriangles that may touch it are visited in submission order and every
 * covered pixel / sample is depth-tested and blended in that order. The
 * reference reaches the same result through a warp-parallel fragment queue
 * (FineRaster.inl:499-752, 855-1126); the conservative culls it applies on
 * the way (early Z, MSAA zslope kill) are checked here instead of applied:
 * or_stats.zmin_violations counts covered samples whose depth falls below
 * the triangle's header zmin, which is the only way those culls could
 * change an output bit.
 */
#include "cr_oracle.h"
#include "shader_math.h"

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef int32_t  S32;
typedef uint32_t U32;
typedef int64_t  S64;
typedef uint64_t U64;
typedef float    F32;

// Constants.hpp:21-46, 81-84
constexpr int SUBPIXEL_LOG2 = 4;
constexpr int TILE_LOG2 = 3;
constexpr int MAXVIEWPORT_LOG2 = 11;  // only used by the fast-path AABB limit
constexpr U32 lerp_error(int s) { return 2200u << s; }
constexpr U32 DEPTH_MIN = 2200u << 3;
constexpr U32 DEPTH_MAX = 0xFFFFFFFFu - (2200u << 3);
constexpr S32 BARY_MAX = (1 << (30 - SUBPIXEL_LOG2)) - 1;
constexpr int FLIP_Y = 2, FLIP_X = 3, SWAP_XY = 4, COMPL = 5;  // Constants.hpp:29-32

// Util.hpp:27-35 -- c_msaaPatterns[log2(samples)][sampleY] = sampleX
const int kMsaaPattern[4][8] = {
    {0},
    {0, 1},
    {1, 3, 0, 2},
    {7, 2, 4, 0, 6, 3, 1, 5},
};

struct F4 { F32 x, y, z, w; };
struct I2 { S32 x, y; };

inline U32 f2u(F32 f) { U32 u; std::memcpy(&u, &f, 4); return u; }
inline S32 f2i(F32 f) { S32 i; std::memcpy(&i, &f, 4); return i; }

// ---- PTX conversion semantics (Util.hpp:88-92 use cvt.*; float->int cvt
// saturates and maps NaN to 0). ----

S32 cvt_rni_sat_s32(F32 a) {  // cvt.rni.sat.s32.f32
    if (std::isnan(a)) return 0;
    if (a >= 2147483648.0f) return INT32_MAX;
    if (a <= -2147483648.0f) return INT32_MIN;
    return (S32)std::nearbyint(a);
}
U32 cvt_rni_sat_u32(F32 a) {  // cvt.rni.sat.u32.f32
    if (!(a > 0.0f)) return 0;
    if (a >= 4294967296.0f) return UINT32_MAX;
    return (U32)std::nearbyint(a);
}
U32 cvt_rmi_sat_u32(F32 a) {  // cvt.rmi.sat.u32.f32
    if (!(a >= 1.0f)) return 0;
    if (a >= 4294967296.0f) return UINT32_MAX;
    return (U32)std::floor(a);
}
S64 cvt_rni_s64(F32 a) {  // cvt.rni.s64.f32
    if (std::isnan(a)) return 0;
    if (a >= 9223372036854775808.0f) return INT64_MAX;
    if (a <= -9223372036854775808.0f) return INT64_MIN;
    return (S64)std::nearbyint(a);
}
U32 cvt_rzi_sat_u32(F32 a) {  // (U32)float on the device: cvt.rzi.u32.f32
    if (!(a >= 1.0f)) return 0;
    if (a >= 4294967296.0f) return UINT32_MAX;
    return (U32)a;
}

// Wrapping integer helpers: the device wraps, C++ would be undefined.
inline S64 wmul64(S64 a, S64 b) { return (S64)((U64)a * (U64)b); }
inline S64 wsub64(S64 a, S64 b) { return (S64)((U64)a - (U64)b); }
inline S64 wadd64(S64 a, S64 b) { return (S64)((U64)a + (U64)b); }
inline S64 sar64(S64 a, S32 n) {  // shr.s64 clamps the shift amount to 64
    if ((U32)n >= 64u) return a < 0 ? -1 : 0;
    return a >> n;
}
inline U32 abs_wrap(S32 v) { return v < 0 ? (U32)0 - (U32)v : (U32)v; }
inline S32 min3(S32 a, S32 b, S32 c) { return std::min(std::min(a, b), c); }
inline S32 max3(S32 a, S32 b, S32 c) { return std::max(std::max(a, b), c); }

// ---- Util.hpp:207-217 cover8x8_selectFlips ----
U32 select_flips(S32 dx, S32 dy) {
    U32 flips = 0;
    if (dy > 0 || (dy == 0 && dx <= 0))
        flips ^= (1u << FLIP_X) ^ (1u << FLIP_Y) ^ (1u << COMPL);
    if (dx > 0)
        flips ^= (1u << FLIP_X) ^ (1u << FLIP_Y);
    if (std::abs((S64)dx) < std::abs((S64)dy))
        flips ^= (1u << SWAP_XY) ^ (1u << FLIP_Y);
    return flips;
}

// ---- Util.hpp:182-203 selectMSAACentroid ----
int select_msaa_centroid(int s, U32 mask) {
    int n = 1 << s;
    if (mask == 0 || mask == (1u << n) - 1) return -1;
    int best = -1, bestDist = INT32_MAX;
    for (int i = 0; i < n; i++) {
        if (mask & (1u << i)) {
            int a = kMsaaPattern[s][i] * 2 + 1 - n;
            int b = i * 2 + 1 - n;
            int d = a * a + b * b;
            if (d < bestDist) { best = i; bestDist = d; }
        }
    }
    return best;
}

// FineRaster.inl:149-164 setupCentroidLUT
U32 centroid_code(int s, U32 mask) {
    U32 value = 0x11u << s;
    int y = select_msaa_centroid(s, mask);
    if (y != -1) value = (U32)(kMsaaPattern[s][y] * 0x02 + y * 0x20 + 0x11);
    return value & 0xFF;
}

// ---- Util.hpp:221-250 clipPolygonWithPlane ----
int clip_polygon(F32* out, const F32* in, int numIn, F32 v0, F32 v1, F32 v2) {
    int numOut = 0;
    if (numIn >= 3) {
        int ai = (numIn - 1) * 2;
        F32 av = v0 + v1 * in[ai + 0] + v2 * in[ai + 1];
        for (int bi = 0; bi < numIn * 2; bi += 2) {
            F32 bv = v0 + v1 * in[bi + 0] + v2 * in[bi + 1];
            if (av * bv < 0.0f) {
                F32 bc = av / (av - bv);
                F32 ac = 1.0f - bc;
                out[numOut + 0] = in[ai + 0] * ac + in[bi + 0] * bc;
                out[numOut + 1] = in[ai + 1] * ac + in[bi + 1] * bc;
                numOut += 2;
            }
            if (bv >= 0.0f) {
                out[numOut + 0] = in[bi + 0];
                out[numOut + 1] = in[bi + 1];
                numOut += 2;
            }
            ai = bi;
            av = bv;
        }
    }
    return numOut >> 1;
}

// ---- Util.hpp:260-286 clipTriangleWithFrustum ----
int clip_triangle(F32* bary, const F32* v0, const F32* v1, const F32* v2,
                  const F32* d1, const F32* d2) {
    int num = 3;
    bary[0] = 0.0f; bary[1] = 0.0f;
    bary[2] = 1.0f; bary[3] = 0.0f;
    bary[4] = 0.0f; bary[5] = 1.0f;
    for (int c = 0; c < 3; c++) {
        if ((v0[3] < std::fabs(v0[c])) | (v1[3] < std::fabs(v1[c])) | (v2[3] < std::fabs(v2[c]))) {
            F32 temp[18];
            num = clip_polygon(temp, bary, num, v0[3] + v0[c], d1[3] + d1[c], d2[3] + d2[c]);
            num = clip_polygon(bary, temp, num, v0[3] - v0[c], d1[3] - d1[c], d2[3] - d2[c]);
        }
    }
    return num;
}

// ---- Util.hpp:290-310 encodeDepth / decodeDepth ----
U32 encode_depth(U32 depth) {
    double v = (double)depth;
    v /= 65536.0 * 65536.0 - 1.0;
    v = std::min(std::max(v, 0.0), 1.0);
    v *= (double)(DEPTH_MAX - DEPTH_MIN);
    v += (double)DEPTH_MIN;
    return (U32)v;
}
U32 decode_depth(U32 depth) {
    double v = (double)depth;
    v -= (double)DEPTH_MIN;
    v *= 1.0 / (double)(DEPTH_MAX - DEPTH_MIN);
    v = std::min(std::max(v, 0.0), 1.0);
    v *= 65536.0 * 65536.0 - 1.0;
    return (U32)v;
}

// ---- Util.inl:30-38 toABGR: byte = cvt.rmi.sat.u32(fma.rm(c, 255*2^24, 2^23)) >> 24.
// The top byte of the round-down result equals clamp(floor(c*255 + 0.5), 0, 255)
// taken exactly (every multiple of 2^24 below 2^32 is a binary32 value), and c*255
// is exact in binary64, so the byte is computed here in binary64. ----
U32 abgr_channel(F32 c) {
    if (std::isnan(c)) return 0;
    double t = std::floor((double)c * 255.0 + 0.5);
    if (t <= 0.0) return 0;
    if (t >= 255.0) return 255;
    return (U32)t;
}
U32 to_abgr(F32 r, F32 g, F32 b, F32 a) {
    return abgr_channel(r) | (abgr_channel(g) << 8) | (abgr_channel(b) << 16) | (abgr_channel(a) << 24);
}

// framework/base/Math.cpp:41-48 Vec4f::toABGR (host side, deferred clear colour)
U32 host_channel(F32 c) {
    F32 cl = std::fmin(std::fmax(c, 0.0f), 1.0f);  // FW::clamp on F32 uses fminf/fmaxf (Defs.hpp:167)
    U64 t = (U64)((double)cl * std::exp2(56.0));
    return (U32)((((t * 255) >> 55) + 1) >> 1);
}
U32 host_to_abgr(F32 r, F32 g, F32 b, F32 a) {
    return host_channel(r) | (host_channel(g) << 8) | (host_channel(b) << 16) | (host_channel(a) << 24);
}

// ---- Util.inl:42-60 blendABGR / blendABGRClamp; PixelPipe.inl:73-85 shaders ----
U32 blend_channel(U32 s, U32 d, U32 sf, U32 df, bool clamp) {
    U32 t = s * sf + d * df;
    if (clamp) t = std::min(t, 255u * 255u);
    return (t * 0x010101u + 0x800000u) >> 24;
}
U32 blend(int mode, U32 src, U32 dst, bool* write) {
    *write = true;
    switch (mode) {
    case OR_BLEND_REPLACE: return src;
    case OR_BLEND_SRCOVER: {
        U32 sa = src >> 24, da = 255u - sa, out = 0;
        for (int c = 0; c < 4; c++)
            out |= blend_channel((src >> (8 * c)) & 0xFF, (dst >> (8 * c)) & 0xFF, sa, da, false) << (8 * c);
        return out;
    }
    case OR_BLEND_ADDITIVE: {
        U32 out = 0;
        for (int c = 0; c < 4; c++)
            out |= blend_channel((src >> (8 * c)) & 0xFF, (dst >> (8 * c)) & 0xFF, 255u, 255u, true) << (8 * c);
        return out;
    }
    default: *write = false; return 0;  // BlendDepthOnly
    }
}

// ---- Util.inl:65-91 setupPleq ----
void setup_pleq(const F32 values[3], I2 v0, I2 d1, I2 d2, F32 areaRcp, int s, U32 out[3]) {
    F32 mx = std::fmax(std::fmax(values[0], values[1]), values[2]);
    int sh = std::min(std::max((f2i(mx) >> 23) - (127 + 22), 0), 8);
    S32 t0 = (S32)(cvt_rzi_sat_u32(values[0]) >> sh);
    S32 t1 = (S32)((cvt_rzi_sat_u32(values[1]) >> sh) - (U32)t0);
    S32 t2 = (S32)((cvt_rzi_sat_u32(values[2]) >> sh) - (U32)t0);

    U32 rcpMant = ((U32)f2i(areaRcp) & 0x007FFFFFu) | 0x00800000u;
    int rcpShift = (23 + 127) - (f2i(areaRcp) >> 23);

    S64 xc = wmul64(wsub64(wmul64(t1, d2.y), wmul64(t2, d1.y)), (S64)rcpMant);
    S64 yc = wmul64(wsub64(wmul64(t2, d1.x), wmul64(t1, d2.x)), (S64)rcpMant);
    out[0] = (U32)sar64(xc, rcpShift - (sh + SUBPIXEL_LOG2 - s));
    out[1] = (U32)sar64(yc, rcpShift - (sh + SUBPIXEL_LOG2 - s));

    S32 centerX = (S32)((U32)v0.x * 2u + (U32)min3(d1.x, d2.x, 0) + (U32)max3(d1.x, d2.x, 0)) >> (SUBPIXEL_LOG2 - s + 1);
    S32 centerY = (S32)((U32)v0.y * 2u + (U32)min3(d1.y, d2.y, 0) + (U32)max3(d1.y, d2.y, 0)) >> (SUBPIXEL_LOG2 - s + 1);
    S32 vcx = (S32)((U32)v0.x - ((U32)centerX << (SUBPIXEL_LOG2 - s)));
    S32 vcy = (S32)((U32)v0.y - ((U32)centerY << (SUBPIXEL_LOG2 - s)));

    U32 z = (U32)t0 << sh;
    z -= (U32)sar64(wadd64(wmul64(sar64(xc, 13), vcx), wmul64(sar64(yc, 13), vcy)), rcpShift - (sh + 13));
    z -= out[0] * (U32)centerX + out[1] * (U32)centerY;
    out[2] = z;
}

struct Header { U32 w[4]; };
struct Data { U32 w[16]; };

struct Viewport {
    S32 width, height;
};

// ---- TriangleSetup.inl:19-31 snapTriangle ----
void snap_triangle(const Viewport& vp, const F4& v0, const F4& v1, const F4& v2,
                   I2& p0, I2& p1, I2& p2, F32 rcpW[3], I2& lo, I2& hi) {
    F32 viewScaleX = (F32)(vp.width << (SUBPIXEL_LOG2 - 1));
    F32 viewScaleY = (F32)(vp.height << (SUBPIXEL_LOG2 - 1));
    rcpW[0] = 1.0f / v0.w;
    rcpW[1] = 1.0f / v1.w;
    rcpW[2] = 1.0f / v2.w;
    p0 = {cvt_rni_sat_s32(v0.x * rcpW[0] * viewScaleX), cvt_rni_sat_s32(v0.y * rcpW[0] * viewScaleY)};
    p1 = {cvt_rni_sat_s32(v1.x * rcpW[1] * viewScaleX), cvt_rni_sat_s32(v1.y * rcpW[1] * viewScaleY)};
    p2 = {cvt_rni_sat_s32(v2.x * rcpW[2] * viewScaleX), cvt_rni_sat_s32(v2.y * rcpW[2] * viewScaleY)};
    lo = {min3(p0.x, p1.x, p2.x), min3(p0.y, p1.y, p2.y)};
    hi = {max3(p0.x, p1.x, p2.x), max3(p0.y, p1.y, p2.y)};
}

// ---- TriangleSetup.inl:38-100 prepareTriangle. 0 visible, 1 backfacing, 2 between samples.
// The area is kept in 64 bits: identical to the reference's S32 product for
// viewports up to 2048 px, and free of overflow above that. ----
int prepare_triangle(const Viewport& vp, int s, I2 p0, I2 p1, I2 p2, I2 lo, I2 hi,
                     I2& d1, I2& d2, S64& area) {
    d1 = {(S32)((U32)p1.x - (U32)p0.x), (S32)((U32)p1.y - (U32)p0.y)};
    d2 = {(S32)((U32)p2.x - (U32)p0.x), (S32)((U32)p2.y - (U32)p0.y)};
    area = (S64)d1.x * d2.y - (S64)d1.y * d2.x;
    if (area <= 0) return 1;

    S32 sampleSize = 1 << (SUBPIXEL_LOG2 - s);
    S32 biasX = (vp.width << (SUBPIXEL_LOG2 - 1)) - (sampleSize >> 1);
    S32 biasY = (vp.height << (SUBPIXEL_LOG2 - 1)) - (sampleSize >> 1);
    S32 lox = (S32)((U32)lo.x + (U32)(sampleSize - 1) + (U32)biasX) & -sampleSize;
    S32 loy = (S32)((U32)lo.y + (U32)(sampleSize - 1) + (U32)biasY) & -sampleSize;
    S32 hix = (S32)((U32)hi.x + (U32)biasX) & -sampleSize;
    S32 hiy = (S32)((U32)hi.y + (U32)biasY) & -sampleSize;
    if (lox > hix || loy > hiy) return 2;

    S32 diff = (S32)((U32)hix + (U32)hiy - (U32)lox - (U32)loy);
    if (diff <= sampleSize) {
        auto edge = [](I2 a, I2 b) { return (S64)a.x * b.y - (S64)a.y * b.x; };
        I2 t0 = {p0.x + biasX - lox, p0.y + biasY - loy};
        I2 t1 = {p1.x + biasX - lox, p1.y + biasY - loy};
        I2 t2 = {p2.x + biasX - lox, p2.y + biasY - loy};
        if (edge(t0, t1) < 0 || edge(t1, t2) < 0 || edge(t2, t0) < 0) {
            if (diff == 0) return 2;
            t0 = {p0.x + biasX - hix, p0.y + biasY - hiy};
            t1 = {p1.x + biasX - hix, p1.y + biasY - hiy};
            t2 = {p2.x + biasX - hix, p2.y + biasY - hiy};
            if (edge(t0, t1) < 0 || edge(t1, t2) < 0 || edge(t2, t0) < 0) return 2;
        }
    }
    return 0;
}

// ---- TriangleSetup.inl:104-215 setupTriangle ----
void setup_triangle(const Viewport& vp, int s, U32 flags, Header& th, Data& td,
                    const S32 vidx[3], const F4& v0, const F4& v1, const F4& v2,
                    const F32 b0[2], const F32 b1[2], const F32 b2[2],
                    I2 p0, I2 p1, I2 p2, const F32 rcpW[3], I2 d1, I2 d2, S64 area) {
    F32 areaRcp = 0.0f;
    I2 wv0 = {0, 0};
    if (flags & (OR_DEPTH | OR_LERP)) {
        areaRcp = 1.0f / (F32)area;
        wv0.x = p0.x + (vp.width << (SUBPIXEL_LOG2 - 1));
        wv0.y = p0.y + (vp.height << (SUBPIXEL_LOG2 - 1));
    }

    U32 zpleq[3] = {0, 0, 0};
    U32 zmin = 0, zslope = 0;
    if (flags & OR_DEPTH) {
        F32 zcoef = (F32)(DEPTH_MAX - DEPTH_MIN) * 0.5f;
        F32 zbias = (F32)(DEPTH_MAX + DEPTH_MIN) * 0.5f;
        F32 zvert[3] = {(v0.z * zcoef) * rcpW[0] + zbias,
                        (v1.z * zcoef) * rcpW[1] + zbias,
                        (v2.z * zcoef) * rcpW[2] + zbias};
        I2 zv0 = {wv0.x - (1 << (SUBPIXEL_LOG2 - s - 1)), wv0.y - (1 << (SUBPIXEL_LOG2 - s - 1))};
        setup_pleq(zvert, zv0, d1, d2, areaRcp, s, zpleq);
        zmin = cvt_rni_sat_u32(std::fmin(std::fmin(zvert[0], zvert[1]), zvert[2]) - (F32)lerp_error(s));
        if (s != 0) {
            U32 tmp = abs_wrap((S32)zpleq[0]) + abs_wrap(std::max((S32)zpleq[1], -INT32_MAX));
            int sh = std::max(s - 1, 0);
            zslope = tmp << sh;
            if ((zslope >> sh) != tmp) zslope = UINT32_MAX;
        }
    }

    U32 wpleq[3] = {0, 0, 0}, upleq[3] = {0, 0, 0}, vpleq[3] = {0, 0, 0};
    if (flags & OR_LERP) {
        F32 wcoef = std::fmin(std::fmin(v0.w, v1.w), v2.w) * (F32)BARY_MAX;
        F32 wvert[3] = {wcoef * rcpW[0], wcoef * rcpW[1], wcoef * rcpW[2]};
        F32 uvert[3] = {b0[0] * wvert[0], b1[0] * wvert[1], b2[0] * wvert[2]};
        F32 vvert[3] = {b0[1] * wvert[0], b1[1] * wvert[1], b2[1] * wvert[2]};
        setup_pleq(wvert, wv0, d1, d2, areaRcp, s + 1, wpleq);
        setup_pleq(uvert, wv0, d1, d2, areaRcp, s + 1, upleq);
        setup_pleq(vvert, wv0, d1, d2, areaRcp, s + 1, vpleq);
    }

    std::memset(&td, 0, sizeof(td));
    if (flags & OR_DEPTH) {
        td.w[0] = zpleq[0]; td.w[1] = zpleq[1]; td.w[2] = zpleq[2]; td.w[3] = zslope;
    }
    if (flags & OR_LERP) {
        td.w[4] = wpleq[0]; td.w[5] = wpleq[1]; td.w[6] = wpleq[2];
        td.w[7] = upleq[0]; td.w[8] = upleq[1]; td.w[9] = upleq[2];
        td.w[10] = vpleq[0]; td.w[11] = vpleq[1]; td.w[12] = vpleq[2];
    }
    td.w[13] = (U32)vidx[0]; td.w[14] = (U32)vidx[1]; td.w[15] = (U32)vidx[2];

    U32 f01 = select_flips(d1.x, d1.y);
    U32 f12 = select_flips(d2.x - d1.x, d2.y - d1.y);
    U32 f20 = select_flips(-d2.x, -d2.y);
    th.w[0] = ((U32)p0.x & 0xFFFFu) | ((U32)p0.y << 16);
    th.w[1] = ((U32)p1.x & 0xFFFFu) | ((U32)p1.y << 16);
    th.w[2] = ((U32)p2.x & 0xFFFFu) | ((U32)p2.y << 16);
    th.w[3] = (zmin & 0xFFFFF000u) | (f01 << 6) | (f12 << 2) | (f20 >> 2);
}

struct Subtri {
    Header h;
    Data d;
};

struct TriSetup {
    int num;          // subtriangles emitted (0..7)
    bool clipped;     // took the clip path
    Subtri sub[7];
};

F4 load_pos(const float* vertices, int stride4, S32 idx) {
    const float* p = vertices + (S64)idx * stride4 * 4;
    return {p[0], p[1], p[2], p[3]};
}

// ---- TriangleSetup.inl:219-417 triangleSetupImpl (one task) ----
void setup_one(const Viewport& vp, int s, U32 flags, const float* vertices, int stride4,
               const S32 vidx[3], TriSetup& out) {
    out.num = 0;
    out.clipped = false;
    F4 v0 = load_pos(vertices, stride4, vidx[0]);
    F4 v1 = load_pos(vertices, stride4, vidx[1]);
    F4 v2 = load_pos(vertices, stride4, vidx[2]);

    if ((v0.w < std::fabs(v0.x)) | (v0.w < std::fabs(v0.y)) | (v0.w < std::fabs(v0.z))) {
        if (((v0.w < +v0.x) & (v1.w < +v1.x) & (v2.w < +v2.x)) |
            ((v0.w < -v0.x) & (v1.w < -v1.x) & (v2.w < -v2.x)) |
            ((v0.w < +v0.y) & (v1.w < +v1.y) & (v2.w < +v2.y)) |
            ((v0.w < -v0.y) & (v1.w < -v1.y) & (v2.w < -v2.y)) |
            ((v0.w < +v0.z) & (v1.w < +v1.z) & (v2.w < +v2.z)) |
            ((v0.w < -v0.z) & (v1.w < -v1.z) & (v2.w < -v2.z)))
            return;
    }

    I2 p0, p1, p2, lo, hi, d1, d2;
    F32 rcpW[3];
    S64 area;
    static const F32 kB0[2] = {0.0f, 0.0f}, kB1[2] = {1.0f, 0.0f}, kB2[2] = {0.0f, 1.0f};

    if ((v0.w >= std::fabs(v0.z)) & (v1.w >= std::fabs(v1.z)) & (v2.w >= std::fabs(v2.z))) {
        snap_triangle(vp, v0, v1, v2, p0, p1, p2, rcpW, lo, hi);
        S32 loxy = std::min(lo.x, lo.y);
        S32 hixy = std::max(hi.x, hi.y);
        S32 aabbLimit = (1 << (MAXVIEWPORT_LOG2 + SUBPIXEL_LOG2)) - 1;
        if (loxy >= -32768 && hixy <= 32767 && hixy - loxy <= aabbLimit) {
            if (prepare_triangle(vp, s, p0, p1, p2, lo, hi, d1, d2, area) == 0) {
                setup_triangle(vp, s, flags, out.sub[0].h, out.sub[0].d, vidx, v0, v1, v2,
                               kB0, kB1, kB2, p0, p1, p2, rcpW, d1, d2, area);
                out.num = 1;
            }
            return;
        }
    }

    // Clip path (TriangleSetup.inl:326-412).
    out.clipped = true;
    F4 ov0 = v0;
    F4 od1 = {v1.x - v0.x, v1.y - v0.y, v1.z - v0.z, v1.w - v0.w};
    F4 od2 = {v2.x - v0.x, v2.y - v0.y, v2.z - v0.z, v2.w - v0.w};
    F32 bary[18];
    int numVerts = clip_triangle(bary, &ov0.x, &v1.x, &v2.x, &od1.x, &od2.x);

    auto lerp = [&](int i) {
        F32 bu = bary[i * 2 + 0], bv = bary[i * 2 + 1];
        return F4{ov0.x + od1.x * bu + od2.x * bv, ov0.y + od1.y * bu + od2.y * bv,
                  ov0.z + od1.z * bu + od2.z * bv, ov0.w + od1.w * bu + od2.w * bv};
    };
    F4 c0 = lerp(0);
    F4 c1 = lerp(1);
    for (int i = 2; i < numVerts; i++) {
        F4 c2 = lerp(i);
        snap_triangle(vp, c0, c1, c2, p0, p1, p2, rcpW, lo, hi);
        if (prepare_triangle(vp, s, p0, p1, p2, lo, hi, d1, d2, area) == 0) {
            F32 b0[2] = {bary[0], bary[1]};
            F32 b1[2] = {bary[i * 2 - 2], bary[i * 2 - 1]};
            F32 b2[2] = {bary[i * 2 + 0], bary[i * 2 + 1]};
            Subtri& st = out.sub[out.num++];
            setup_triangle(vp, s, flags, st.h, st.d, vidx, c0, c1, c2, b0, b1, b2,
                           p0, p1, p2, rcpW, d1, d2, area);
        }
        c1 = c2;
    }
}

// ---- Coverage: exact edge functions with the fill rule (Util.inl:95-102,
// 340-357). o = vertex relative to the sample, d = edge direction. ----
inline bool edge_covers(S64 ox, S64 oy, S64 dx, S64 dy) {
    S64 e = ox * dy - oy * dx;
    if (dy > 0 || (dy == 0 && dx <= 0)) e--;
    return e >= 0;
}

struct TriGeom {
    S32 v0x, v0y, v1x, v1y, v2x, v2y;  // subpixels relative to the viewport centre
};

TriGeom geom_from_header(const Header& h) {
    TriGeom g;
    g.v0x = (int16_t)(h.w[0] & 0xFFFF); g.v0y = (int16_t)(h.w[0] >> 16);
    g.v1x = (int16_t)(h.w[1] & 0xFFFF); g.v1y = (int16_t)(h.w[1] >> 16);
    g.v2x = (int16_t)(h.w[2] & 0xFFFF); g.v2y = (int16_t)(h.w[2] >> 16);
    return g;
}

// Sample point (px, py) in the header's frame, covered by the triangle?
// FineRaster.inl:244-305: edges (v0, v1-v0), (v1, v2-v1), (v0, v0-v2).
inline bool tri_covers(const TriGeom& g, S64 px, S64 py) {
    return edge_covers(g.v0x - px, g.v0y - py, (S64)g.v1x - g.v0x, (S64)g.v1y - g.v0y) &&
           edge_covers(g.v1x - px, g.v1y - py, (S64)g.v2x - g.v1x, (S64)g.v2y - g.v1y) &&
           edge_covers(g.v0x - px, g.v0y - py, (S64)g.v0x - g.v2x, (S64)g.v0y - g.v2y);
}

// MSAA sample offsets in subpixels (Util.inl:361-367).
inline S32 sample_dx(int s, int i) { return s == 0 ? 0 : (kMsaaPattern[s][i] * 2 + 1 - (1 << s)) << (SUBPIXEL_LOG2 - s - 1); }
inline S32 sample_dy(int s, int i) { return s == 0 ? 0 : (i * 2 + 1 - (1 << s)) << (SUBPIXEL_LOG2 - s - 1); }

// Pixel centre of pixel x in the header frame: (x << 4) - ((W - 1) << 3).
inline S64 pixel_cx(const Viewport& vp, S64 x) { return (x << SUBPIXEL_LOG2) - ((S64)(vp.width - 1) << (SUBPIXEL_LOG2 - 1)); }
inline S64 pixel_cy(const Viewport& vp, S64 y) { return (y << SUBPIXEL_LOG2) - ((S64)(vp.height - 1) << (SUBPIXEL_LOG2 - 1)); }

U32 sample_mask(const Viewport& vp, int s, const TriGeom& g, S32 x, S32 y) {
    S64 cx = pixel_cx(vp, x), cy = pixel_cy(vp, y);
    U32 m = 0;
    for (int i = 0; i < (1 << s); i++)
        if (tri_covers(g, cx + sample_dx(s, i), cy + sample_dy(s, i))) m |= 1u << i;
    return m;
}

// ---- FineRaster.inl:21-44 computeBarys ----
struct Barys { F32 c[3], dx[3], dy[3]; };

Barys compute_barys(int s, const S32 w[3], const S32 u[3], const S32 v[3], S32 sx, S32 sy) {
    auto ev = [&](const S32 p[3]) { return (S32)((U32)p[0] * (U32)sx + (U32)p[1] * (U32)sy + (U32)p[2]); };
    Barys b;
    F32 wr = 1.0f / (F32)ev(w);
    F32 uu = wr * (F32)ev(u);
    F32 vv = wr * (F32)ev(v);
    b.c[0] = 1.0f - uu - vv; b.c[1] = uu; b.c[2] = vv;
    F32 wd = wr * (F32)(1 << (s + 1));
    F32 udx = wd * ((F32)u[0] - uu * (F32)w[0]);
    F32 udy = wd * ((F32)u[1] - uu * (F32)w[1]);
    F32 vdx = wd * ((F32)v[0] - vv * (F32)w[0]);
    F32 vdy = wd * ((F32)v[1] - vv * (F32)w[1]);
    b.dx[0] = -udx - vdx; b.dx[1] = udx; b.dx[2] = vdx;
    b.dy[0] = -udy - vdy; b.dy[1] = udy; b.dy[2] = vdy;
    return b;
}

// ---- Fragment shaders ----
struct ShadeCtx {
    const float* vertices;
    int stride4;
    int s;
    U32 flags;
    int shader;
};

// PixelPipe.inl:43-59 interpolateVarying (varying k of vertex i at vertices[i*stride + 1 + k]).
void interpolate(const ShadeCtx& c, const Data& d, int k, const F32 bary[3], F32 out[4]) {
    const float* a = c.vertices + ((S64)d.w[13] * c.stride4 + 1 + k) * 4;
    const float* b = c.vertices + ((S64)d.w[14] * c.stride4 + 1 + k) * 4;
    const float* e = c.vertices + ((S64)d.w[15] * c.stride4 + 1 + k) * 4;
    for (int i = 0; i < 4; i++) out[i] = a[i] * bary[0] + b[i] * bary[1] + e[i] * bary[2];
}

U32 trihash_color(S32 triIdx) {
    U32 h = (U32)triIdx * 2654435761u;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    return h | 0xFF000000u;
}

using crsm::evaluate_lighting;
using crsm::log2_full;
using crsm::pow_exact;
using crsm::tex2d;

// The textured Phong shader's inputs (the reference's c_constants and
// t_textureAtlas). Materials are the reference's 576-byte Material records.
struct TexPhongEnv {
    const F32* materials = nullptr;  // 144 floats each
    int numMaterials = 0;
    const int32_t* triMaterial = nullptr;
    S64 numTriMaterial = 0;
    const U32* atlas = nullptr;
    S32 atlasW = 0, atlasH = 0;
};
TexPhongEnv g_texPhong;

// Shaders.cu:123-147 texture2D; spec = the TextureSpec's 68 floats (size, pad, mip levels).
void texture2d(const F32* spec, const F32 tex[2], const F32 texDX[2], const F32 texDY[2], F32 out[4]) {
    const F32 sx = spec[0], sy = spec[1];
    const F32 ax = texDX[0] * sx, ay = texDX[1] * sy, bx = texDY[0] * sx, by = texDY[1] * sy;
    const F32 dxlen = ax * ax + ay * ay;
    const F32 dylen = bx * bx + by * by;
    const F32 lod = std::fmin(std::fmax(log2_full(std::fmax(dxlen, dylen)) * 0.5f, 0.0f), 14.0f);
    const int levelIdx = (int)lod;
    const F32* m0 = spec + 4 + 4 * levelIdx;
    const F32* m1 = m0 + 4;
    const F32 tx = tex[0] - std::floor(tex[0]);
    const F32 ty = tex[1] - std::floor(tex[1]);
    F32 v0[4], v1[4];
    const TexPhongEnv& e = g_texPhong;
    tex2d(e.atlas, e.atlasW, e.atlasH, tx * m0[0] + m0[2], ty * m0[1] + m0[3], v0);
    tex2d(e.atlas, e.atlasW, e.atlasH, tx * m1[0] + m1[2], ty * m1[1] + m1[3], v1);
    const F32 t = lod - (F32)levelIdx;
    const F32 omt = 1.0f - t;
    for (int k = 0; k < 4; k++) out[k] = v0[k] * omt + v1[k] * t;
}

// test/shader/Shaders.cu:149-193 FragmentShader_texPhong::run. Without quads
// the texture is sampled at the centroid with its analytic derivatives; in
// quad mode at the pixel centre, with dFdx / dFdy the differences of the
// pixel-centre values across the 2x2 quad (right minus left in the row,
// bottom minus top in the column).
U32 shade_tex_phong(const ShadeCtx& c, const Data& d, S32 triIdx, S32 px, S32 py, const Barys& cb, bool* discard) {
    F32 cp[4], cn[4], tex[2], texDX[2], texDY[2];
    interpolate(c, d, 0, cb.c, cp);
    interpolate(c, d, 1, cb.c, cn);
    if (!(c.flags & OR_QUADS)) {
        F32 t[4], tdx[4], tdy[4];
        interpolate(c, d, 2, cb.c, t);
        interpolate(c, d, 2, cb.dx, tdx);
        interpolate(c, d, 2, cb.dy, tdy);
        tex[0] = t[0]; tex[1] = t[1];
        texDX[0] = tdx[0]; texDX[1] = tdx[1];
        texDY[0] = tdy[0]; texDY[1] = tdy[1];
    } else {
        const S32 w[3] = {(S32)d.w[4], (S32)d.w[5], (S32)d.w[6]};
        const S32 u[3] = {(S32)d.w[7], (S32)d.w[8], (S32)d.w[9]};
        const S32 v[3] = {(S32)d.w[10], (S32)d.w[11], (S32)d.w[12]};
        auto texAt = [&](S32 qx, S32 qy, F32 out[4]) {
            Barys b = compute_barys(c.s, w, u, v, (qx * 2 + 1) << c.s, (qy * 2 + 1) << c.s);
            interpolate(c, d, 2, b.c, out);
        };
        const S32 x0 = px & ~1, y0 = py & ~1;
        F32 t[4], l[4], r[4], tp[4], bt[4];
        texAt(px, py, t);
        texAt(x0, py, l);
        texAt(x0 + 1, py, r);
        texAt(px, y0, tp);
        texAt(px, y0 + 1, bt);
        tex[0] = t[0]; tex[1] = t[1];
        texDX[0] = r[0] - l[0]; texDX[1] = r[1] - l[1];
        texDY[0] = bt[0] - tp[0]; texDY[1] = bt[1] - tp[1];
    }
    const TexPhongEnv& e = g_texPhong;
    if (!e.materials || !e.triMaterial || !e.atlas || e.numMaterials < 1 || e.numTriMaterial < 1) {
        *discard = true;  // no inputs set: as the GPU shader, nothing to read
        return 0;
    }
    const S64 slot = std::min((S64)triIdx, e.numTriMaterial - 1);
    const int materialIdx = std::min(std::max((int)e.triMaterial[slot], 0), e.numMaterials - 1);
    const F32* m = e.materials + (S64)materialIdx * 144;
    F32 diffuse[4] = {m[0], m[1], m[2], m[3]};
    const F32* diffuseTexture = m + 8;
    const F32* alphaTexture = m + 76;
    F32 tc[4];
    if (diffuseTexture[0] != 0.0f) {
        texture2d(diffuseTexture, tex, texDX, texDY, tc);
        diffuse[0] = tc[0]; diffuse[1] = tc[1]; diffuse[2] = tc[2];
    }
    if (alphaTexture[0] != 0.0f) {
        texture2d(alphaTexture, tex, texDX, texDY, tc);
        diffuse[3] = tc[1];
    }
    if (diffuse[3] < 0.5f) {
        *discard = true;
        return 0;
    }
    F32 color[3];
    evaluate_lighting(cp, cn, m + 4, m[7], diffuse, color);
    return to_abgr(color[0], color[1], color[2], diffuse[3]);
}

// FineRaster.inl:48-119 runFragmentShader, for the shaders the oracle knows.
U32 shade(const ShadeCtx& c, const Data& d, S32 triIdx, S32 px, S32 py, U32 centroid, bool* discard) {
    *discard = false;
    F32 center[3] = {0.0f, 0.0f, 1.0f}, centroidB[3] = {0.0f, 0.0f, 1.0f};
    Barys bc{}, cb{};  // at the pixel centre, at the centroid (with derivatives)
    cb.c[2] = 1.0f;
    if (c.flags & OR_LERP) {
        const S32 w[3] = {(S32)d.w[4], (S32)d.w[5], (S32)d.w[6]};
        const S32 u[3] = {(S32)d.w[7], (S32)d.w[8], (S32)d.w[9]};
        const S32 v[3] = {(S32)d.w[10], (S32)d.w[11], (S32)d.w[12]};
        bc = compute_barys(c.s, w, u, v, (px * 2 + 1) << c.s, (py * 2 + 1) << c.s);
        std::memcpy(center, bc.c, sizeof(center));
        if (c.s == 0) {
            cb = bc;
        } else {
            cb = compute_barys(c.s, w, u, v, (px << (c.s + 1)) + (S32)(centroid & 0xF),
                               (py << (c.s + 1)) + (S32)(centroid >> 4));
        }
        std::memcpy(centroidB, cb.c, sizeof(centroidB));
    }
    switch (c.shader) {
    case OR_SHADER_GOURAUD: {
        F32 col[4];
        interpolate(c, d, 0, centroidB, col);
        return to_abgr(col[0], col[1], col[2], col[3]);
    }
    case OR_SHADER_RED:
        return to_abgr(1.0f, 0.0f, 0.0f, 1.0f);
    case OR_SHADER_TRIHASH:
        return trihash_color(triIdx);
    case OR_SHADER_TEXPHONG:
        return shade_tex_phong(c, d, triIdx, px, py, cb, discard);
    default:
        return to_abgr(bc.dx[1] * 64.0f, bc.dy[1] * 64.0f, center[2], 1.0f);
    }
}

// The test pipe's derivative shader in quad mode (its GPU twin reads the
// interpolated v barycentric u = m_center.y): colour = (|dFdx u| * 64,
// |dFdy u| * 64, m_center.z, 1), the differences taken across the 2x2 quad
// of pixel (x, y) between pixel-centre barycentrics.
U32 shade_deriv_quad(const ShadeCtx& c, const Data& d, S32 x, S32 y) {
    const S32 w[3] = {(S32)d.w[4], (S32)d.w[5], (S32)d.w[6]};
    const S32 u[3] = {(S32)d.w[7], (S32)d.w[8], (S32)d.w[9]};
    const S32 v[3] = {(S32)d.w[10], (S32)d.w[11], (S32)d.w[12]};
    auto bary = [&](S32 qx, S32 qy) { return compute_barys(c.s, w, u, v, (qx * 2 + 1) << c.s, (qy * 2 + 1) << c.s); };
    const S32 x0 = x & ~1, y0 = y & ~1;
    const F32 dx = bary(x0 + 1, y).c[1] - bary(x0, y).c[1];
    const F32 dy = bary(x, y0 + 1).c[1] - bary(x, y0).c[1];
    return to_abgr(std::fabs(dx) * 64.0f, std::fabs(dy) * 64.0f, bary(x, y).c[2], 1.0f);
}

inline S64 row_words(const or_pipe* p) {
    S64 rw = ((S64)p->width + 7) & ~7LL;
    return rw << p->samples_log2;
}
inline S64 surface_index(const or_pipe* p, S32 x, S32 y, int i) {
    return (S64)y * row_words(p) + (S64)(x >> 3) * (8 << p->samples_log2) + i * 8 + (x & 7);
}

}  // namespace

namespace {
struct QItem { U32 entry; TriGeom g; };

bool edge_touches_rect(S64 ox, S64 oy, S64 dx, S64 dy, S64 rx0, S64 ry0, S64 rx1, S64 ry1) {
    S64 px = dy > 0 ? rx0 : rx1;
    S64 py = dx > 0 ? ry1 : ry0;
    return (ox - px) * dy - (oy - py) * dx >= 0;
}

bool tri_touches_rect(const TriGeom& g, S64 rx0, S64 ry0, S64 rx1, S64 ry1) {
    return edge_touches_rect(g.v0x, g.v0y, g.v1x - g.v0x, g.v1y - g.v0y, rx0, ry0, rx1, ry1) &&
           edge_touches_rect(g.v1x, g.v1y, g.v2x - g.v1x, g.v2y - g.v1y, rx0, ry0, rx1, ry1) &&
           edge_touches_rect(g.v2x, g.v2y, g.v0x - g.v2x, g.v0y - g.v2y, rx0, ry0, rx1, ry1);
}

// Cells of the rule in the window [wx0, wx1] x [wy0, wy1] of a grid with cells
// of 2^cellLog2 subpixels.
template <class Fn>
void rule_cells(const Viewport& vp, int samplesLog2, const TriGeom& g, int cellLog2, S32 wx0, S32 wy0, S32 wx1,
                S32 wy1, Fn fn) {
    const S32 hw = vp.width << (SUBPIXEL_LOG2 - 1), hh = vp.height << (SUBPIXEL_LOG2 - 1);
    // One sample per pixel: the box of the pixel centres (16 p + 8 from the
    // viewport's edge) inside the vertex box; with MSAA the vertex box.
    const S32 lo = samplesLog2 == 0 ? 7 : 0, hi = samplesLog2 == 0 ? 8 : 0;
    S32 lx = std::max((min3(g.v0x, g.v1x, g.v2x) + hw + lo) >> cellLog2, wx0);
    S32 hx = std::min((max3(g.v0x, g.v1x, g.v2x) + hw - hi) >> cellLog2, wx1);
    S32 ly = std::max((min3(g.v0y, g.v1y, g.v2y) + hh + lo) >> cellLog2, wy0);
    S32 hy = std::min((max3(g.v0y, g.v1y, g.v2y) + hh - hi) >> cellLog2, wy1);
    if (lx > hx || ly > hy) return;
    const bool small = hx - lx <= 1 && hy - ly <= 1;
    const S64 side = (S64)1 << cellLog2;
    for (S32 cy = ly; cy <= hy; cy++)
        for (S32 cx = lx; cx <= hx; cx++) {
            const S64 rx0 = ((S64)cx << cellLog2) - hw, ry0 = ((S64)cy << cellLog2) - hh;
            if (small || tri_touches_rect(g, rx0, ry0, rx0 + side - 1, ry0 + side - 1)) fn(cx, cy);
        }
}
}  // namespace

// ===================================================================== C API

extern "C" {

int64_t or_setup(const or_pipe* p, const float* vertices, const int32_t* indices,
                 int64_t num_tris, uint8_t* tri_subtris, uint32_t* headers,
                 uint32_t* data, int64_t max_subtris) {
    Viewport vp{p->width, p->height};
    int stride4 = p->vertex_stride / 16;
    std::vector<TriSetup> res((size_t)std::max<int64_t>(num_tris, 0));
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < num_tris; t++)
        setup_one(vp, p->samples_log2, p->render_mode, vertices, stride4, &indices[t * 3], res[t]);
    int64_t next = num_tris;
    for (int64_t t = 0; t < num_tris; t++) {
        const TriSetup& r = res[t];
        tri_subtris[t] = (uint8_t)r.num;
        if (r.num == 1) {
            std::memcpy(&headers[t * 4], r.sub[0].h.w, 16);
            std::memcpy(&data[t * 16], r.sub[0].d.w, 64);
        } else if (r.num > 1) {
            if (next + r.num > max_subtris) return -1;
            headers[t * 4 + 3] = (uint32_t)next;
            for (int i = 0; i < r.num; i++) {
                std::memcpy(&headers[(next + i) * 4], r.sub[i].h.w, 16);
                std::memcpy(&data[(next + i) * 16], r.sub[i].d.w, 64);
            }
            next += r.num;
        }
    }
    return next;
}

int or_render(const or_pipe* p, const float* vertices, const int32_t* indices,
              int64_t num_tris, uint32_t* color, uint32_t* depth,
              int num_threads, or_stats* stats) {
#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#endif
    Viewport vp{p->width, p->height};
    const int s = p->samples_log2;
    const int ns = 1 << s;
    const int stride4 = p->vertex_stride / 16;
    const S32 wTiles = (p->width + 7) >> 3, hTiles = (p->height + 7) >> 3;

    // Setup (TriangleSetup.inl), parallel over triangles.
    std::vector<TriSetup> res((size_t)std::max<int64_t>(num_tris, 0));
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < num_tris; t++)
        setup_one(vp, s, p->render_mode, vertices, stride4, &indices[t * 3], res[t]);

    // Flat subtriangle list in submission order with tile-space bounding boxes.
    struct Item { int64_t tri; int sub; S32 tx0, ty0, tx1, ty1; };
    std::vector<Item> items;
    int64_t clipped = 0;
    for (int64_t t = 0; t < num_tris; t++) {
        clipped += res[t].clipped ? 1 : 0;
        for (int i = 0; i < res[t].num; i++) {
            TriGeom g = geom_from_header(res[t].sub[i].h);
            S32 cx = p->width << (SUBPIXEL_LOG2 - 1), cy = p->height << (SUBPIXEL_LOG2 - 1);
            S32 lx = min3(g.v0x, g.v1x, g.v2x) + cx, hx = max3(g.v0x, g.v1x, g.v2x) + cx;
            S32 ly = min3(g.v0y, g.v1y, g.v2y) + cy, hy = max3(g.v0y, g.v1y, g.v2y) + cy;
            int sh = SUBPIXEL_LOG2 + TILE_LOG2;
            Item it{t, i, std::max(lx >> sh, 0), std::max(ly >> sh, 0),
                    std::min(hx >> sh, wTiles - 1), std::min(hy >> sh, hTiles - 1)};
            if (it.tx0 <= it.tx1 && it.ty0 <= it.ty1) items.push_back(it);
        }
    }

    int64_t numSub = 0;
    for (int64_t t = 0; t < num_tris; t++) numSub += res[t].num;

    // Bin by tile rows: each thread owns a band of tile rows.
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
    int64_t frags = 0, violations = 0, entries = 0;
    ShadeCtx sc{vertices, stride4, s, p->render_mode, p->shader};
    const bool useDepth = (p->render_mode & OR_DEPTH) != 0;

#pragma omp parallel num_threads(nthreads) reduction(+ : frags, violations, entries)
    {
        int tid = 0, nt = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        // Tile rows are interleaved over threads (row ty belongs to thread
        // ty % nt); every thread walks the item list in submission order and
        // keeps the entries of its own rows, so each tile list stays ordered.
        std::vector<std::vector<std::vector<int32_t>>> rowLists;
        std::vector<S32> myRows;
        for (S32 ty = tid; ty < hTiles; ty += nt) myRows.push_back(ty);
        rowLists.resize(myRows.size());
        for (auto& r : rowLists) r.resize(wTiles);
        for (size_t k = 0; k < items.size(); k++) {
            const Item& it = items[k];
            S32 first = it.ty0 + (((tid - it.ty0) % nt) + nt) % nt;
            for (S32 ty = first; ty <= it.ty1; ty += nt) {
                size_t r = (size_t)(ty / nt);
                for (S32 tx = it.tx0; tx <= it.tx1; tx++) rowLists[r][tx].push_back((int32_t)k);
            }
        }
        std::vector<U32> tc(64 * ns), td(64 * ns);
        for (size_t r = 0; r < myRows.size(); r++) {
            S32 ty = myRows[r];
            for (S32 tx = 0; tx < wTiles; tx++) {
                const std::vector<int32_t>& list = rowLists[r][tx];
                if (list.empty() && !p->deferred_clear) continue;
                entries += (int64_t)list.size();
                // Load or clear the tile (FineRaster.inl:562-580, 916-929).
                for (int py = 0; py < 8; py++)
                    for (int px = 0; px < 8; px++)
                        for (int i = 0; i < ns; i++) {
                            S64 idx = surface_index(p, tx * 8 + px, ty * 8 + py, i);
                            int k = (py * 8 + px) * ns + i;
                            tc[k] = p->deferred_clear ? p->clear_color : color[idx];
                            td[k] = p->deferred_clear ? p->clear_depth : depth[idx];
                        }
                for (int32_t li : list) {
                    const Item& it = items[(size_t)li];
                    const Subtri& st = res[(size_t)it.tri].sub[it.sub];
                    TriGeom g = geom_from_header(st.h);
                    const U32 zmin = st.h.w[3] & 0xFFFFF000u;
                    // Quad mode (FineRaster.inl:401-427): a 2x2 quad is shaded when
                    // any of its pixels is covered; its uncovered pixels are helpers
                    // that only feed the derivatives (PixelPipe.hpp:62-69: dFdx is
                    // the right minus the left pixel of the row, dFdy the bottom
                    // minus the top pixel of the column).
                    const bool quads = (p->render_mode & OR_QUADS) != 0;
                    for (int pi = 0; pi < 64; pi++) {
                        int px, py;
                        if (quads) {
                            const int q = pi >> 2, k = pi & 3;
                            px = ((q & 3) << 1) + (k & 1);
                            py = ((q >> 2) << 1) + (k >> 1);
                        } else {
                            px = pi & 7;
                            py = pi >> 3;
                        }
                        {
                            S32 x = tx * 8 + px, y = ty * 8 + py;
                            U32 mask = sample_mask(vp, s, g, x, y);
                            if (mask == 0) continue;
                            frags++;
                            int base = (py * 8 + px) * ns;
                            // Per-sample depth (FineRaster.inl:695, 1047, 1096).
                            U32 dz[8];
                            bool anyPass = !useDepth;
                            for (int i = 0; i < ns; i++) {
                                if (s == 0)
                                    dz[i] = st.d.w[0] * (U32)x + st.d.w[1] * (U32)y + st.d.w[2];
                                else
                                    dz[i] = st.d.w[0] * (U32)kMsaaPattern[s][i] + st.d.w[1] * (U32)i +
                                            (((st.d.w[0] * (U32)x + st.d.w[1] * (U32)y) << s) + st.d.w[2]);
                                if (useDepth && (mask >> i & 1)) {
                                    if (dz[i] < zmin) violations++;
                                    if (dz[i] < td[base + i]) anyPass = true;
                                }
                            }
                            if (!anyPass) continue;
                            bool discard;
                            U32 src;
                            if (quads && p->shader == OR_SHADER_DERIV)
                                src = shade_deriv_quad(sc, st.d, x, y);
                            else
                                src = shade(sc, st.d, (S32)it.tri, x, y, centroid_code(s, mask), &discard);
                            discard = quads && p->shader == OR_SHADER_DERIV ? false : discard;
                            if (discard) continue;
                            for (int i = 0; i < ns; i++) {
                                if (!(mask >> i & 1)) continue;
                                if (useDepth) {
                                    if (!(dz[i] < td[base + i])) continue;
                                    td[base + i] = dz[i];
                                }
                                bool wr;
                                U32 out = blend(p->blend, src, tc[base + i], &wr);
                                if (wr) tc[base + i] = out;
                            }
                        }
                    }
                }
                for (int py = 0; py < 8; py++)
                    for (int px = 0; px < 8; px++)
                        for (int i = 0; i < ns; i++) {
                            S64 idx = surface_index(p, tx * 8 + px, ty * 8 + py, i);
                            int k = (py * 8 + px) * ns + i;
                            color[idx] = tc[k];
                            depth[idx] = td[k];
                        }
            }
        }
    }
    if (stats) {
        stats->num_subtris = numSub;
        stats->num_clipped = clipped;
        stats->num_fragments = frags;
        stats->zmin_violations = violations;
        stats->tile_entries = entries;
    }
    return 0;
}

// Per-stage queue model: the bin and tile lists of one draw, by cell, as
// CSR arrays. Entries are triangle << 3 | subtriangle (7 when the triangle has
// one subtriangle: BinRaster.inl:148-158), in submission order.
//   kind 0 / 2: bins / tiles, exact -- entries covering at least one sample of
//               the cell's pixels (the per-sample rule above);
//   kind 1 / 3: bins / tiles, the binning rule of the GPU stages -- the
//               entry's bounding box (at one sample per pixel the box of the
//               pixel centres inside it), in cells and clamped to the cell window
//               (the viewport's bins; for tiles the tiles of the bin), contains
//               the cell, and either the clamped box spans at most 2x2 cells or
//               no edge has the whole cell rectangle strictly outside; a tile
//               only takes entries of its bin's list. The reference bins
//               conservatively in the same sense (BinRaster.inl:228-300,
//               CoarseRaster.inl:299-435).
// Fills offsets[num_cells + 1] and entries[] when the total fits `cap`;
// returns the total (-1 on bad arguments).

int64_t or_queue_lists(const or_pipe* p, const float* vertices, const int32_t* indices, int64_t num_tris,
                       int bin_log2, int kind, int64_t* offsets, uint32_t* entries, int64_t cap) {
    if (bin_log2 < 3 || bin_log2 > 5 || kind < 0 || kind > 3) return -1;
    Viewport vp{p->width, p->height};
    const int s = p->samples_log2;
    const int stride4 = p->vertex_stride / 16;
    std::vector<TriSetup> res((size_t)std::max<int64_t>(num_tris, 0));
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < num_tris; t++)
        setup_one(vp, s, p->render_mode, vertices, stride4, &indices[t * 3], res[t]);
    std::vector<QItem> items;
    for (int64_t t = 0; t < num_tris; t++)
        for (int i = 0; i < res[t].num; i++)
            items.push_back({(U32)(t << 3) | (U32)(res[t].num == 1 ? 7 : i), geom_from_header(res[t].sub[i].h)});
    const S32 wt = (p->width + 7) >> 3, ht = (p->height + 7) >> 3;
    const S32 side = 1 << bin_log2;
    const S32 wb = (wt + side - 1) / side, hb = (ht + side - 1) / side;
    const bool bins = kind < 2, exact = (kind & 1) == 0;
    const S64 numCells = bins ? (S64)wb * hb : (S64)wt * ht;
    std::vector<std::vector<U32>> lists((size_t)numCells);
    const int tileCell = SUBPIXEL_LOG2 + TILE_LOG2, binCell = tileCell + bin_log2;
    for (const QItem& it : items) {
        if (exact) {
            // Every tile whose pixels hold a covered sample (boxes clamped to the viewport's tiles).
            const S32 hw = vp.width << (SUBPIXEL_LOG2 - 1), hh = vp.height << (SUBPIXEL_LOG2 - 1);
            S32 lx = std::max((min3(it.g.v0x, it.g.v1x, it.g.v2x) + hw) >> tileCell, 0);
            S32 hx = std::min((max3(it.g.v0x, it.g.v1x, it.g.v2x) + hw) >> tileCell, wt - 1);
            S32 ly = std::max((min3(it.g.v0y, it.g.v1y, it.g.v2y) + hh) >> tileCell, 0);
            S32 hy = std::min((max3(it.g.v0y, it.g.v1y, it.g.v2y) + hh) >> tileCell, ht - 1);
            for (S32 ty = ly; ty <= hy; ty++)
                for (S32 tx = lx; tx <= hx; tx++) {
                    bool hit = false;
                    for (int pi = 0; pi < 64 && !hit; pi++)
                        hit = sample_mask(vp, s, it.g, tx * 8 + (pi & 7), ty * 8 + (pi >> 3)) != 0;
                    if (!hit) continue;
                    if (!bins) {
                        lists[(size_t)ty * wt + tx].push_back(it.entry);
                    } else {
                        std::vector<U32>& l = lists[(size_t)(ty >> bin_log2) * wb + (tx >> bin_log2)];
                        if (l.empty() || l.back() != it.entry) l.push_back(it.entry);
                    }
                }
        } else {
            rule_cells(vp, s, it.g, binCell, 0, 0, wb - 1, hb - 1, [&](S32 bx, S32 by) {
                if (bins) {
                    lists[(size_t)by * wb + bx].push_back(it.entry);
                    return;
                }
                const S32 x0 = bx << bin_log2, y0 = by << bin_log2;
                rule_cells(vp, s, it.g, tileCell, x0, y0, std::min(x0 + side - 1, wt - 1), std::min(y0 + side - 1, ht - 1),
                           [&](S32 tx, S32 ty) { lists[(size_t)ty * wt + tx].push_back(it.entry); });
            });
        }
    }
    if (exact && bins)
        for (auto& l : lists) {   // an entry's tiles of one bin are not consecutive in row order
            std::sort(l.begin(), l.end());
            l.erase(std::unique(l.begin(), l.end()), l.end());
        }
    int64_t total = 0;
    for (const auto& l : lists) total += (int64_t)l.size();
    if (total <= cap && offsets && (entries || total == 0)) {
        int64_t o = 0;
        for (S64 c = 0; c < numCells; c++) {
            offsets[c] = o;
            for (U32 e : lists[(size_t)c]) entries[o++] = e;
        }
        offsets[numCells] = o;
    }
    return total;
}

int32_t or_f32_to_s32_sat(float a) { return cvt_rni_sat_s32(a); }
uint32_t or_f32_to_u32_sat(float a) { return cvt_rni_sat_u32(a); }
uint32_t or_f32_to_u32_sat_rmi(float a) { return cvt_rmi_sat_u32(a); }
int64_t or_f32_to_s64(float a) { return cvt_rni_s64(a); }
uint32_t or_f32_to_u32_rz(float a) { return cvt_rzi_sat_u32(a); }
uint32_t or_to_abgr(float r, float g, float b, float a) { return to_abgr(r, g, b, a); }
uint32_t or_host_to_abgr(float r, float g, float b, float a) { return host_to_abgr(r, g, b, a); }
uint32_t or_encode_depth(uint32_t d) { return encode_depth(d); }
uint32_t or_decode_depth(uint32_t d) { return decode_depth(d); }

// CudaRaster.cpp:178 deferredClear depth encoding.
uint32_t or_clear_depth(float depth) {
    double v = (double)depth * std::exp2(32.0);
    U64 t;
    if (!(v > 0.0)) t = 0;
    else if (v >= 18446744073709551616.0) t = UINT64_MAX;
    else t = (U64)v;
    return encode_depth((U32)std::min<U64>(t, 0xFFFFFFFFull));
}

uint32_t or_blend(int mode, uint32_t src, uint32_t dst, int* write_color) {
    bool w;
    U32 r = blend(mode, src, dst, &w);
    if (write_color) *write_color = w ? 1 : 0;
    return r;
}
uint32_t or_select_flips(int32_t dx, int32_t dy) { return select_flips(dx, dy); }
int or_select_msaa_centroid(int s, uint32_t mask) { return select_msaa_centroid(s, mask); }
void or_centroid_lut(int s, uint8_t* lut) {
    for (U32 m = 0; m < (1u << (1 << s)); m++) lut[m] = (uint8_t)centroid_code(s, m);
}
void or_setup_pleq(const float values[3], const int32_t v0[2], const int32_t d1[2],
                   const int32_t d2[2], float area_rcp, int s, uint32_t out[3]) {
    setup_pleq(values, I2{v0[0], v0[1]}, I2{d1[0], d1[1]}, I2{d2[0], d2[1]}, area_rcp, s, out);
}
int or_clip_triangle(float* bary18, const float v0[4], const float v1[4], const float v2[4],
                     const float d1[4], const float d2[4]) {
    return clip_triangle(bary18, v0, v1, v2, d1, d2);
}

// Util.inl:95-134 cover8x8_exact_ref / conservative_ref (bit i <-> pixel (i&7, i>>3)).
static uint64_t cover8x8(S64 curr, S64 stepX, S64 stepY) {
    uint64_t m = 0;
    for (int i = 0; i < 64; i++) {
        S64 v = curr + (i & 7) * stepX + (i >> 3) * stepY;
        if (v >= 0) m |= 1ull << i;
    }
    return m;
}
uint64_t or_cover8x8_exact(int32_t ox, int32_t oy, int32_t dx, int32_t dy) {
    S64 curr = (S64)ox * dy - (S64)oy * dx;
    S64 stepX = -(S64)dy * 16, stepY = (S64)dx * 16;
    if (dy > 0 || (dy == 0 && dx <= 0)) curr--;
    return cover8x8(curr, stepX, stepY);
}
uint64_t or_cover8x8_conservative(int32_t ox, int32_t oy, int32_t dx, int32_t dy) {
    S64 curr = (S64)ox * dy - (S64)oy * dx;
    S64 stepX = -(S64)dy * 16, stepY = (S64)dx * 16;
    if (dy > 0 || (dy == 0 && dx <= 0)) curr--;
    curr += (std::llabs(stepX) + std::llabs(stepY)) >> 1;
    return cover8x8(curr, stepX, stepY);
}
// Util.inl:340-357 coverMSAA_ref
uint32_t or_cover_msaa(int s, int32_t ox, int32_t oy, int32_t dx, int32_t dy) {
    U32 m = 0;
    for (int i = 0; i < (1 << s); i++)
        if (edge_covers((S64)ox - sample_dx(s, i), (S64)oy - sample_dy(s, i), dx, dy)) m |= 1u << i;
    return m;
}

// FineRaster.inl:244-280 trianglePixelCoverage (exact for 1 sample, conservative otherwise).
uint64_t or_triangle_pixel_coverage(const uint32_t header[4], int tile_x, int tile_y,
                                    int width, int height, int s) {
    Header h;
    std::memcpy(h.w, header, 16);
    TriGeom g = geom_from_header(h);
    Viewport vp{width, height};
    S64 bx = pixel_cx(vp, (S64)tile_x * 8), by = pixel_cy(vp, (S64)tile_y * 8);
    S64 v0x = g.v0x - bx, v0y = g.v0y - by;
    S64 e[3][4] = {{v0x, v0y, (S64)g.v1x - g.v0x, (S64)g.v1y - g.v0y},
                   {g.v1x - bx, g.v1y - by, (S64)g.v2x - g.v1x, (S64)g.v2y - g.v1y},
                   {v0x, v0y, (S64)g.v0x - g.v2x, (S64)g.v0y - g.v2y}};
    uint64_t m = ~0ull;
    for (int k = 0; k < 3; k++) {
        S64 curr = e[k][0] * e[k][3] - e[k][1] * e[k][2];
        S64 stepX = -e[k][3] * 16, stepY = e[k][2] * 16;
        if (e[k][3] > 0 || (e[k][3] == 0 && e[k][2] <= 0)) curr--;
        if (s != 0) curr += (std::llabs(stepX) + std::llabs(stepY)) >> 1;
        m &= cover8x8(curr, stepX, stepY);
    }
    return m;
}
// FineRaster.inl:284-305 triangleSampleCoverage
uint32_t or_triangle_sample_coverage(const uint32_t header[4], int px, int py,
                                     int width, int height, int s) {
    Header h;
    std::memcpy(h.w, header, 16);
    return sample_mask(Viewport{width, height}, s, geom_from_header(h), px, py);
}
void or_compute_barys(int s, const int32_t w[3], const int32_t u[3], const int32_t v[3],
                      int32_t sx, int32_t sy, float out[9]) {
    Barys b = compute_barys(s, w, u, v, sx, sy);
    std::memcpy(out, b.c, 12);
    std::memcpy(out + 3, b.dx, 12);
    std::memcpy(out + 6, b.dy, 12);
}
// FineRaster.inl:341-399 findBit
int or_find_bit(uint64_t mask, int idx, int quads) {
    if (!quads) {
        for (int row = 0; row < 8; row++) {
            U32 r = (U32)(mask >> (row * 8)) & 0xFF;
            int pop = __builtin_popcount(r);
            if (idx < pop) {
                for (int b = 7; b >= 0; b--)
                    if (r >> b & 1) { if (idx == 0) return row * 8 + b; idx--; }
            }
            idx -= pop;
        }
        return -1;
    }
    for (int b = 0; b < 64; b++)
        if (mask >> b & 1) { if (idx == 0) return b; idx--; }
    return -1;
}
void or_set_tex_phong(const float* materials, int num_materials, const int32_t* triangle_material_idx,
                      int64_t num_triangle_material_idx, const uint32_t* atlas, int atlas_width, int atlas_height) {
    g_texPhong.materials = materials;
    g_texPhong.numMaterials = num_materials;
    g_texPhong.triMaterial = triangle_material_idx;
    g_texPhong.numTriMaterial = num_triangle_material_idx;
    g_texPhong.atlas = atlas;
    g_texPhong.atlasW = atlas_width;
    g_texPhong.atlasH = atlas_height;
}

void or_texture_sample(const uint32_t* atlas, int atlas_width, int atlas_height, const float* uv, float* out,
                       int64_t n) {
    for (int64_t i = 0; i < n; i++) tex2d(atlas, atlas_width, atlas_height, uv[2 * i], uv[2 * i + 1], out + 4 * i);
}

// The GPU filter's division-free form of s / (255 * 65536) (ShaderMath.hpp
// crTexNormalize) against the division the specification states, for every
// weighted sum s the filter can form; returns the number of differences.
int64_t or_tex_normalize_mismatches(void) {
    const F32 rcp = 0.00392156886f;
    int64_t bad = 0;
    for (U32 s = 0; s <= 16711680u; s++) {
        const F32 x = (F32)s;
        const F32 q0 = x * rcp;
        const F32 r = std::fmaf(-q0, 255.0f, x);
        const F32 q = std::fmaf(r, rcp, q0);
        if (q * 1.52587890625e-05f != x / 16711680.0f) bad++;
    }
    return bad;
}

float or_pow_exact(float x, float y) { return pow_exact(x, y); }
float or_log2_exact(float x) { return log2_full(x); }

void or_evaluate_lighting(const float camera_pos[3], const float camera_normal[3], const float specular[3],
                          float glossiness, const float diffuse[3], float out[3]) {
    evaluate_lighting(camera_pos, camera_normal, specular, glossiness, diffuse, out);
}

uint32_t or_fragment(const or_pipe* p, const uint32_t data16[16], const float* vertices,
                     int32_t tri_idx, int32_t px, int32_t py, uint32_t centroid) {
    ShadeCtx c{vertices, p->vertex_stride / 16, p->samples_log2, p->render_mode, p->shader};
    Data d;
    std::memcpy(d.w, data16, 64);
    bool discard;
    return shade(c, d, tri_idx, px, py, centroid, &discard);
}

// framework/base/Math.cpp:75-88 Mat4f::perspective (row-major out).
void or_perspective(float fov, float n, float f, float out[16]) {
    F32 t = std::tan(fov * 3.14159265358979323846f / 360.0f);  // binary32 tan
    F32 fv = (t != 0.0f) ? 1.0f / t : 0.0f;                    // rcp (Math.hpp:113)
    F32 d = 1.0f / (n - f);
    std::memset(out, 0, 64);
    out[0] = fv;
    out[5] = fv;
    out[10] = (n + f) * d;
    out[11] = 2.0f * n * f * d;
    out[14] = -1.0f;
}

}  // extern "C"
