// cr_device.cuh -- data layouts, per-draw descriptors and the fixed-point /
// floating-point arithmetic shared by the GB300 pipeline kernels.
//
// Arithmetic follows the reference's device code operation by operation
// (tcoppex/cudaraster-linux src/cudaraster/cuda/*.inl). Every binary32
// operation that the reference writes as an expression is issued here as an
// explicitly rounded intrinsic (__fmul_rn, __fadd_rn, ...), so no FMA
// contraction can change a bit whatever flags a translation unit is built
// with. Float->integer conversions use the saturating cvt forms the
// reference's inline PTX uses (Util.hpp:88-92).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cr {

typedef int32_t S32;
typedef uint32_t U32;
typedef int64_t S64;
typedef uint64_t U64;
typedef float F32;

// Constants.hpp:21-46, 81-84
constexpr int kSubpixelLog2 = 4;
constexpr int kTileLog2 = 3;
constexpr int kMaxViewportLog2Ref = 11;  // fast-path AABB limit of TriangleSetup.inl:294
constexpr U32 kDepthMin = 2200u << 3;
constexpr U32 kDepthMax = 0xFFFFFFFFu - (2200u << 3);
constexpr S32 kBaryMax = (1 << (30 - kSubpixelLog2)) - 1;
__host__ __device__ constexpr U32 lerpError(int s) { return 2200u << s; }
constexpr int kFlipY = 2, kFlipX = 3, kSwapXY = 4, kCompl = 5;

enum : U32 {
    kRenderDepth = 1u,
    kRenderLerp = 2u,
    kRenderQuads = 4u,
};

// Overflow flags raised on the device and read back by the host rerun loop.
enum : int {
    kOverflowSubtris = 1,
    kOverflowBin = 2,
    kOverflowTile = 4,
};

// ---------------------------------------------------------------- layouts
// CRTriangleHeader (PrivateDefs.hpp:26-36): 3 x (S16 x, S16 y) in subpixels
// relative to the viewport centre + misc = (zmin:20 | f01:4 | f12:4 | f20:4),
// or the first slot of the subtriangles when a clipped triangle emits > 1.
// CRTriangleData (PrivateDefs.hpp:40-62): zx zy zb zslope | wx wy wb | ux uy
// ub | vx vy vb | vi0 vi1 vi2, 16 words.

// Per-scene descriptor (one per instance of a batch; one for a plain draw).
struct InstanceDev {
    const float4* vertices;   // vertex records, stride4 float4 each
    const int* indices;       // 3 ints per triangle
    U32* color;               // surfaces (reference layout)
    U32* depth;
    S64 rowWords;             // (roundedWidth << samplesLog2)
    S32 stride4;              // vertex record size in float4 units
    S32 numTris;
    S32 width, height;        // viewport
    S32 widthTiles, heightTiles;
    S32 widthBins, heightBins;
    S32 samplesLog2;
    S32 deferredClear;
    U32 clearColor, clearDepth;
    S64 triBase;              // first triangle slot of this instance
    S32 binBase;              // first global bin id
    S32 tileBase;             // first global tile id
    S32 chunkBase;            // first global bin-stage chunk
    S32 numChunks;
    S64 chunkCountBase;       // first entry of this instance in chunkBinCount / chunkBinOffset
    S32 chunkTris;            // triangles per chunk
    S32 pipeGroup;            // index of the pipe this instance renders with
};

struct Counters {
    S32 extraSubtris;         // subtriangle slots allocated past the triangle slots
    S32 binEntries;           // total bin list entries
    S32 numUnits;             // coarse work units
    S32 tileEntries;          // total tile list entries
    S32 fineTile;             // fine-stage work counter
    S32 overflow;             // kOverflow* bits
    S32 coarseWork[2];        // coarse count / scatter unit counters (dynamic unit assignment)
    S32 binWork[2];           // bin count / scatter chunk counters (dynamic chunk assignment)
    S32 binsDone;             // bin-scan CTAs finished (the last one plans the coarse units)
    S32 unitEntries;          // bin entries per coarse unit, as planned for this draw
};

// Buffers shared by every instance of a draw.
struct DrawDev {
    const InstanceDev* inst;  // [numInstances]
    S32 numInstances;
    S32 binLog2;              // tiles per bin side (log2)
    S32 totalBins;
    S32 totalTiles;
    S32 totalChunks;
    S32 maxBins;              // bins of the largest instance
    S32 fineSelfPixels;       // fine stage: pixel-box size up to which a lane rasterizes a triangle alone
    S32 unitEntries;          // bin entries per coarse unit; <= 0: sized on the device from the bin entries
    S32 unitTarget;           // coarse units wanted when sized on the device (set by the launcher)
    S64 totalTris;
    // Fused vertex transform (single draws): when model is set, setup takes a
    // vertex's clip position as mvp * (model[i], 1) -- the reference's
    // vertexShader_passthrough -- instead of reading the record's clipPos.
    const float* model;       // xyz at modelStride floats per vertex, or null
    S32 modelStride;
    S32 modelVec4;            // stride 4 and 16-byte aligned: one vector load per vertex
    F32 mvp[16];              // row-major
    // setup
    uint8_t* triSubtris;      // [totalTris]
    uint4* triHeader;         // [maxSubtris]
    uint4* triData;           // [maxSubtris * 4]
    S32* subtriOwner;         // [maxSubtris - totalTris] triangle of an extra slot
    S64 maxSubtris;
    // bin
    S32* chunkBinCount;       // per (bin, chunk): entry count; zero between draws (the bin scan clears it)
    S32* chunkBinOffset;      // per (chunk, bin): exclusive offset of the chunk in the bin list
    S32* binCount;            // [totalBins]
    S32* binStart;            // [totalBins]
    S32* binUnitFirst;        // [totalBins]
    U32* binList;             // [maxBinEntries]
    S64 maxBinEntries;
    // coarse
    S32* unitTileCount;       // [maxUnits << 2*binLog2]: count, then offset
    S64 maxUnits;
    S32* tileCount;           // [totalTiles]
    S32* tileStart;           // [totalTiles]
    U32* tileList;            // [maxTileEntries]
    S64 maxTileEntries;
    // instance lookup tables (prefix sums, numInstances + 1 entries)
    const S32* chunkPrefix;   // chunks
    const S32* binPrefix;     // bins
    const S32* tilePrefix;    // tiles
    const S64* triPrefix;     // triangles
    Counters* counters;
    S32* fineTileCounter;     // [pipe groups] fine-stage tile work counters
    // Pairs recorded by the bin count pass for the bin scatter pass: chunk c's
    // (bin << 32 | list entry) pairs in list order at binStage[c * binStageCap],
    // their number in binStageCount[c]. A chunk with more pairs than
    // binStageCap (or binStageCap 0) is walked again by the scatter pass.
    U64* binStage;
    S32* binStageCount;       // [totalChunks]
    S32 binStageCap;
    // Likewise for the coarse passes: unit u < tileStageUnits records its
    // (tile of the bin << 32 | list entry) pairs at tileStage[u * tileStageCap].
    U64* tileStage;
    S32* tileStageCount;      // [tileStageUnits]
    S32 tileStageCap;
    S32 tileStageUnits;
    // Device address of the pinned host copy of the counters: the draw's first
    // fine launch writes them there (every stage that changes them has
    // finished by then), in place of a device-to-host copy after the draw.
    // Null in every other launch.
    Counters* hostCounters;
};

// ------------------------------------------------------ instance lookup
// Largest i with prefix[i] <= v (prefix has n + 1 ascending entries).
__device__ __forceinline__ int findInstance(const S32* prefix, int n, S32 v) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&prefix[mid]) <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int findInstance64(const S64* prefix, int n, S64 v) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&prefix[mid]) <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ------------------------------------------------------------- arithmetic
__device__ __forceinline__ S32 f32_to_s32_sat(F32 a) { return __float2int_rn(a); }       // cvt.rni.sat.s32.f32
__device__ __forceinline__ U32 f32_to_u32_sat(F32 a) { return __float2uint_rn(a); }      // cvt.rni.sat.u32.f32
__device__ __forceinline__ U32 f32_to_u32_sat_rmi(F32 a) { return __float2uint_rd(a); }  // cvt.rmi.sat.u32.f32
__device__ __forceinline__ U32 f32_to_u32_rz(F32 a) { return __float2uint_rz(a); }       // (U32)float
__device__ __forceinline__ F32 fmul(F32 a, F32 b) { return __fmul_rn(a, b); }
__device__ __forceinline__ F32 fadd(F32 a, F32 b) { return __fadd_rn(a, b); }
__device__ __forceinline__ F32 fsub(F32 a, F32 b) { return __fsub_rn(a, b); }
__device__ __forceinline__ F32 fdiv(F32 a, F32 b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ F32 frcp(F32 a) { return __frcp_rn(a); }  // 1 / a, correctly rounded (= __fdiv_rn(1, a))
__device__ __forceinline__ S32 min3i(S32 a, S32 b, S32 c) { return min(min(a, b), c); }
__device__ __forceinline__ S32 max3i(S32 a, S32 b, S32 c) { return max(max(a, b), c); }
// shr.s64 semantics: shift amounts >= 64 give the sign fill.
__device__ __forceinline__ S64 sar64(S64 a, S32 n) { return ((U32)n >= 64u) ? (a >> 63) : (a >> n); }
__device__ __forceinline__ U32 absWrap(S32 v) { return v < 0 ? 0u - (U32)v : (U32)v; }

// toABGR (Util.inl:30-38): fma.rm then cvt.rmi.sat.u32, top byte.
__device__ __forceinline__ U32 toABGR(F32 r, F32 g, F32 b, F32 a) {
    const F32 scale = (F32)(1 << 24) * 255.0f, bias = (F32)(1 << 24) * 0.5f;
    U32 x = f32_to_u32_sat_rmi(__fmaf_rd(r, scale, bias)) >> 24;
    U32 y = f32_to_u32_sat_rmi(__fmaf_rd(g, scale, bias)) >> 24;
    U32 z = f32_to_u32_sat_rmi(__fmaf_rd(b, scale, bias)) >> 24;
    U32 w = f32_to_u32_sat_rmi(__fmaf_rd(a, scale, bias)) >> 24;
    return x | (y << 8) | (z << 16) | (w << 24);
}

// blendABGR / blendABGRClamp (Util.inl:42-60): per channel
// ((s * sf + d * df) * 0x010101 + 0x800000) >> 24 with 8-bit factors.
__device__ __forceinline__ U32 blendChannels(U32 src, U32 dst, U32 sf, U32 df, U32 saf, U32 daf, bool clamp) {
    U32 out = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        U32 s = (src >> (8 * c)) & 0xFF, d = (dst >> (8 * c)) & 0xFF;
        U32 t = (c < 3) ? (s * sf + d * df) : (s * saf + d * daf);
        if (clamp) t = min(t, 255u * 255u);
        out |= ((t * 0x010101u + 0x800000u) >> 24) << (8 * c);
    }
    return out;
}

// selectFlips (Util.hpp:207-217)
__device__ __forceinline__ U32 selectFlips(S32 dx, S32 dy) {
    U32 flips = 0;
    if (dy > 0 || (dy == 0 && dx <= 0)) flips ^= (1u << kFlipX) ^ (1u << kFlipY) ^ (1u << kCompl);
    if (dx > 0) flips ^= (1u << kFlipX) ^ (1u << kFlipY);
    if (abs(dx) < abs(dy)) flips ^= (1u << kSwapXY) ^ (1u << kFlipY);
    return flips;
}

// setupPleq (Util.inl:65-91). v0 = subpixels relative to the first sample.
__device__ __forceinline__ void setupPleq(F32 vx, F32 vy, F32 vz, int2 v0, int2 d1, int2 d2,
                                          F32 areaRcp, int s, U32& ox, U32& oy, U32& oz) {
    F32 mx = fmaxf(fmaxf(vx, vy), vz);
    int sh = min(max((__float_as_int(mx) >> 23) - (127 + 22), 0), 8);
    S32 t0 = (S32)(f32_to_u32_rz(vx) >> sh);
    S32 t1 = (S32)((f32_to_u32_rz(vy) >> sh) - (U32)t0);
    S32 t2 = (S32)((f32_to_u32_rz(vz) >> sh) - (U32)t0);
    U32 rcpMant = ((U32)__float_as_int(areaRcp) & 0x007FFFFFu) | 0x00800000u;
    int rcpShift = (23 + 127) - (__float_as_int(areaRcp) >> 23);
    S64 xc = (S64)((U64)((S64)t1 * d2.y - (S64)t2 * d1.y) * (U64)rcpMant);
    S64 yc = (S64)((U64)((S64)t2 * d1.x - (S64)t1 * d2.x) * (U64)rcpMant);
    ox = (U32)sar64(xc, rcpShift - (sh + kSubpixelLog2 - s));
    oy = (U32)sar64(yc, rcpShift - (sh + kSubpixelLog2 - s));
    S32 centerX = (S32)((U32)v0.x * 2u + (U32)min3i(d1.x, d2.x, 0) + (U32)max3i(d1.x, d2.x, 0)) >> (kSubpixelLog2 - s + 1);
    S32 centerY = (S32)((U32)v0.y * 2u + (U32)min3i(d1.y, d2.y, 0) + (U32)max3i(d1.y, d2.y, 0)) >> (kSubpixelLog2 - s + 1);
    S32 vcx = (S32)((U32)v0.x - ((U32)centerX << (kSubpixelLog2 - s)));
    S32 vcy = (S32)((U32)v0.y - ((U32)centerY << (kSubpixelLog2 - s)));
    U32 z = (U32)t0 << sh;
    U64 cross = (U64)sar64(xc, 13) * (U64)(S64)vcx + (U64)sar64(yc, 13) * (U64)(S64)vcy;
    z -= (U32)sar64((S64)cross, rcpShift - (sh + 13));
    z -= ox * (U32)centerX + oy * (U32)centerY;
    oz = z;
}

// clipPolygonWithPlane (Util.hpp:221-250), unfused.
__device__ __forceinline__ int clipPolygon(F32* out, const F32* in, int numIn, F32 v0, F32 v1, F32 v2) {
    int numOut = 0;
    if (numIn >= 3) {
        int ai = (numIn - 1) * 2;
        F32 av = fadd(fadd(v0, fmul(v1, in[ai + 0])), fmul(v2, in[ai + 1]));
        for (int bi = 0; bi < numIn * 2; bi += 2) {
            F32 bv = fadd(fadd(v0, fmul(v1, in[bi + 0])), fmul(v2, in[bi + 1]));
            if (fmul(av, bv) < 0.0f) {
                F32 bc = fdiv(av, fsub(av, bv));
                F32 ac = fsub(1.0f, bc);
                out[numOut + 0] = fadd(fmul(in[ai + 0], ac), fmul(in[bi + 0], bc));
                out[numOut + 1] = fadd(fmul(in[ai + 1], ac), fmul(in[bi + 1], bc));
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

// clipTriangleWithFrustum (Util.hpp:260-286)
__device__ __forceinline__ int clipTriangle(F32* bary, const F32* v0, const F32* v1, const F32* v2,
                                            const F32* d1, const F32* d2) {
    int num = 3;
    bary[0] = 0.0f; bary[1] = 0.0f;
    bary[2] = 1.0f; bary[3] = 0.0f;
    bary[4] = 0.0f; bary[5] = 1.0f;
#pragma unroll 1
    for (int c = 0; c < 3; c++) {
        if ((v0[3] < fabsf(v0[c])) | (v1[3] < fabsf(v1[c])) | (v2[3] < fabsf(v2[c]))) {
            F32 temp[18];
            num = clipPolygon(temp, bary, num, fadd(v0[3], v0[c]), fadd(d1[3], d1[c]), fadd(d2[3], d2[c]));
            num = clipPolygon(bary, temp, num, fsub(v0[3], v0[c]), fsub(d1[3], d1[c]), fsub(d2[3], d2[c]));
        }
    }
    return num;
}

// MSAA sample offsets in subpixels relative to the pixel centre
// (Util.hpp:27-35 patterns, Util.inl:361-367 placement).
__host__ __device__ constexpr int msaaPatternX(int s, int i) {
    return s == 0 ? 0
         : s == 1 ? (i == 0 ? 0 : 1)
         : s == 2 ? (i == 0 ? 1 : i == 1 ? 3 : i == 2 ? 0 : 2)
         : (i == 0 ? 7 : i == 1 ? 2 : i == 2 ? 4 : i == 3 ? 0 : i == 4 ? 6 : i == 5 ? 3 : i == 6 ? 1 : 5);
}
__host__ __device__ constexpr int sampleOffsetX(int s, int i) {
    return s == 0 ? 0 : (msaaPatternX(s, i) * 2 + 1 - (1 << s)) << (kSubpixelLog2 - s - 1);
}
__host__ __device__ constexpr int sampleOffsetY(int s, int i) {
    return s == 0 ? 0 : (i * 2 + 1 - (1 << s)) << (kSubpixelLog2 - s - 1);
}

// selectMSAACentroid (Util.hpp:182-203) + setupCentroidLUT (FineRaster.inl:149-164).
__device__ __forceinline__ U32 centroidCode(int s, U32 mask) {
    int n = 1 << s;
    if (mask == 0 || mask == (1u << n) - 1) return (0x11u << s) & 0xFF;
    int best = -1, bestDist = 0x7FFFFFFF;
    for (int i = 0; i < n; i++) {
        if (mask & (1u << i)) {
            int a = msaaPatternX(s, i) * 2 + 1 - n, b = i * 2 + 1 - n;
            int d = a * a + b * b;
            if (d < bestDist) { best = i; bestDist = d; }
        }
    }
    return (U32)(msaaPatternX(s, best) * 0x02 + best * 0x20 + 0x11) & 0xFF;
}

__device__ __forceinline__ S32 lo16(U32 v) { return (S32)(int16_t)(uint16_t)(v & 0xFFFF); }
__device__ __forceinline__ S32 hi16(U32 v) { return (S32)(int16_t)(uint16_t)(v >> 16); }

}  // namespace cr
