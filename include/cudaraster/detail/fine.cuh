// fine.cuh -- fine raster kernel (stage 4 of 4).
//
// One warp owns one 8x8 tile at a time (persistent warps pulling tiles from a
// counter, as FineRaster.inl:534-552). The tile's colour and depth live in the
// warp's shared memory for the whole tile. Its triangle list is consumed in
// batches of 32; lane i fetches entry i (header, data slot, early-Z against
// the tile's current maximum depth as FineRaster.inl:229-240, edge functions
// at the tile origin). Then one of two algorithms runs, chosen at compile time:
//
// Both paths deal the (triangle, pixel) pairs of the batch's small triangles
// (pixel box of at most fineSelfPixels pixels) over the lanes; larger
// triangles are rasterized by the 32 pixel-owning lanes, two pixels each.
//
// Ordered path (any blend shader, discard, quads):
//   coverage masks per triangle (set by the pairs, or by ballots over the
//   pixel-owning lanes for large triangles), covered pixels compacted into
//   passes of 32 fragments in submission order (FineRaster.inl:625-731), then
//   depth test, shading and blending per fragment. Fragments of one pass that
//   hit the same pixel are grouped with __match_any_sync and applied one rank
//   at a time in lane order, which is submission order. This replaces the
//   reference's reliance on lock-step warps for same-address shared-memory
//   races (FineRaster.inl:433-495, 758-851), undefined on sm_70 and later.
//   With one sample, a depth test and a fragment shader that never discards,
//   a fragment later in the batch than its pixel's minimum (depth, then
//   position) is dropped before compaction: it would fail the LESS test.
//
// Visibility path (depth test on, blend shader that ignores the destination,
//   fragment shader that never discards): the final colour and depth of a
//   sample are those of its front-most covering fragment, the earliest one in
//   submission order on equal depth -- the same result as applying every
//   fragment in order with a LESS test. Each sample keeps a 64-bit key
//   (depth << 32 | list position + 1) that fragments lower with atomicMin;
//   after the list, the tile's winners are listed and each is shaded once,
//   32 at a time.
//
// MSAA keeps every sample of the tile in shared memory (reference layout:
// sample i of pixel x at word i * 8 + x of the tile row) and shades once per
// (pixel, triangle) at the centroid of the triangle's covered samples.
#pragma once

#include "../PixelPipe.hpp"
#include "device.cuh"
#include "launch.h"

#include <type_traits>

namespace cr {

constexpr int kFineMaxThreads = 256;
// Triangles whose pixel box inside the tile has at most DrawDev::fineSelfPixels
// pixels are rasterized pixel by pixel by the lanes -- their (triangle, pixel)
// pairs are dealt over all lanes; larger ones by the whole warp, two
// pixels per lane. Default: 16 pixels.
__host__ __device__ constexpr int fineSelfPixelsDefault(int, bool) { return 16; }


// The ordered path's per-warp state (one warp per tile).
template <int S>
struct FineWarpSmem {
    static constexpr int kTileWords = 64 << S;
    U32 color[kTileWords];
    U32 depth[kTileWords];
    U32 pairBox[32];       // bx0 | by0 << 4 | w << 8 of each small triangle's pixel box
    U32 pairMul[32];       // ceil(2^16 / w)
    S32 E[3][32];          // edge functions at the tile's pixel (0, 0) centre, bias folded in
    S32 A[3][32];          // per-subpixel x step (-dy)
    S32 B[3][32];          // per-subpixel y step (+dx)
    U32 td[16][32];        // triangle data slots (CRTriangleData words)
    S32 tri[32];           // triangle index within the draw
    U32 covLo[32];
    U32 covHi[32];
    // One sample, depth test on, no discard: each pixel's minimum of
    // (depth << 32 | batch triangle) over the batch's covered fragments.
    U64 batchMin[S == 0 ? 64 : 1];
    S32 fragEnd[32];       // inclusive prefix of the small triangles' pair counts
    S32 fragHead[32];      // batch triangle whose fragments start at position i of the current pass
    F32 shared[32];
};

// A triangle of the visibility path's batch in 12 words: edge functions
// E0-2, A0-2, B0-2 (see TileEdges) and depth plane zx, zy, zb. Lanes read a
// record with three 128-bit loads: all lanes the same one (a broadcast) on
// the large-triangle path; on the pair path lanes of a quarter warp read
// consecutive records, whose 48-byte stride puts any eight of them on
// distinct banks.
struct TriRec {
    uint4 q[3];   // E0 E1 E2 A0 | A1 A2 B0 B1 | B2 zx zy zb
};

// The visibility path's per-warp state: no separate depth array (a key's high
// word is its sample's depth) and only the triangle words it reads.
template <int S>
struct FineVisSmem {
    static constexpr int kTileWords = 64 << S;
    U32 color[kTileWords];
    U64 key[kTileWords];        // depth << 32 | order (order << 8 | coverage mask with MSAA)
    TriRec rec[32];             // the batch's triangles
    U32 box[32];                // bx0 | by0 << 4 | w << 8 | ceil(2^16 / w) << 12: a small triangle's pixel box
    S32 head[32];               // batch triangle whose pairs start at position i of the current pass
    U32 winners[kTileWords];    // resolve: (pixel | first sample << 6 | samples won << 9)
    F32 shared[32];
};

// Compile-time shape of a pipe's fine stage.
template <class FS, class BS, int S, U32 F>
struct FineTraits {
    static constexpr bool kDepth = (F & kRenderDepth) != 0;
    static constexpr bool kQuads = (F & kRenderQuads) != 0;
    // Opaque depth-tested pipes resolve visibility with keys (see fineKernel).
    static constexpr bool kVisibility = kDepth && !kQuads && !FW::BlendShaderTraits<BS>::needsDst &&
                                        !FW::FragmentShaderTraits<FS>::mayDiscard;
    using Smem = typename std::conditional<kVisibility, FineVisSmem<S>, FineWarpSmem<S>>::type;
};

__device__ __forceinline__ int nthSetBit32(U32 m, int n) {
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        U32 lowMask = (1u << w) - 1u;
        int c = __popc(m & lowMask);
        if (n >= c) { n -= c; m >>= w; pos += w; }
    }
    return pos;
}
__device__ __forceinline__ int nthSetBit64(U32 lo, U32 hi, int n) {
    int c = __popc(lo);
    return (n < c) ? nthSetBit32(lo, n) : 32 + nthSetBit32(hi, n - c);
}

// computeBarys (FineRaster.inl:21-44)
template <int S>
__device__ __forceinline__ void computeBarys(FW::Vec3f& b, FW::Vec3f& bdx, FW::Vec3f& bdy, const U32* w,
                                             const U32* u, const U32* v, S32 sx, S32 sy) {
    F32 wr = frcp(__int2float_rn((S32)(w[0] * (U32)sx + w[1] * (U32)sy + w[2])));
    F32 uu = fmul(wr, __int2float_rn((S32)(u[0] * (U32)sx + u[1] * (U32)sy + u[2])));
    F32 vv = fmul(wr, __int2float_rn((S32)(v[0] * (U32)sx + v[1] * (U32)sy + v[2])));
    b = FW::Vec3f(fsub(fsub(1.0f, uu), vv), uu, vv);
    F32 wd = fmul(wr, (F32)(1 << (S + 1)));
    F32 udx = fmul(wd, fsub(__int2float_rn((S32)u[0]), fmul(uu, __int2float_rn((S32)w[0]))));
    F32 udy = fmul(wd, fsub(__int2float_rn((S32)u[1]), fmul(uu, __int2float_rn((S32)w[1]))));
    F32 vdx = fmul(wd, fsub(__int2float_rn((S32)v[0]), fmul(vv, __int2float_rn((S32)w[0]))));
    F32 vdy = fmul(wd, fsub(__int2float_rn((S32)v[1]), fmul(vv, __int2float_rn((S32)w[1]))));
    bdx = FW::Vec3f(fsub(-udx, vdx), udx, vdx);
    bdy = FW::Vec3f(fsub(-udy, vdy), udy, vdy);
}

__device__ __forceinline__ S32 clampEdge(S64 e) {
    const S64 lim = (S64)1 << 30;
    return (S32)(e > lim ? lim : (e < -lim ? -lim : e));
}

// Edge functions of a header relative to the tile's pixel (0, 0) centre:
// edges (v0, v1 - v0), (v1, v2 - v1), (v0, v0 - v2) as FineRaster.inl:251-275,
// bias of the fill rule (Util.inl:100) folded in. A sample at subpixel offset
// q from that centre is covered iff E[k] + A[k] * q.x + B[k] * q.y >= 0 for
// all k (the offsets stay below 2^8 and |A|, |B| below 2^17, so clamping E to
// +-2^30 keeps every sign).
struct TileEdges {
    S32 E[3], A[3], B[3];
    S32 minX, maxX, minY, maxY;   // vertex box relative to the pixel (0, 0) centre
};

__device__ __forceinline__ TileEdges tileEdges(uint4 h, S32 cx0, S32 cy0) {
    TileEdges t;
    S32 vx[3] = {lo16(h.x) - cx0, lo16(h.y) - cx0, lo16(h.z) - cx0};
    S32 vy[3] = {hi16(h.x) - cy0, hi16(h.y) - cy0, hi16(h.z) - cy0};
    const int oi[3] = {0, 1, 0};
    S32 ddx[3] = {vx[1] - vx[0], vx[2] - vx[1], vx[0] - vx[2]};
    S32 ddy[3] = {vy[1] - vy[0], vy[2] - vy[1], vy[0] - vy[2]};
#pragma unroll
    for (int k = 0; k < 3; k++) {
        S64 e = (S64)vx[oi[k]] * ddy[k] - (S64)vy[oi[k]] * ddx[k];
        if (ddy[k] > 0 || (ddy[k] == 0 && ddx[k] <= 0)) e -= 1;
        t.E[k] = clampEdge(e);
        t.A[k] = -ddy[k];
        t.B[k] = ddx[k];
    }
    t.minX = min3i(vx[0], vx[1], vx[2]);
    t.maxX = max3i(vx[0], vx[1], vx[2]);
    t.minY = min3i(vy[0], vy[1], vy[2]);
    t.maxY = max3i(vy[0], vy[1], vy[2]);
    return t;
}

__device__ __forceinline__ bool edgesCover(const S32* E, const S32* A, const S32* B, S32 qx, S32 qy) {
    return (E[0] + A[0] * qx + B[0] * qy >= 0) && (E[1] + A[1] * qx + B[1] * qy >= 0) &&
           (E[2] + A[2] * qx + B[2] * qy >= 0);
}

// Exact sample mask of pixel (px, py) of the tile.
template <int S>
__device__ __forceinline__ U32 sampleMaskOf(const S32* E, const S32* A, const S32* B, S32 px, S32 py) {
    U32 m = 0;
#pragma unroll
    for (int i = 0; i < (1 << S); i++)
        if (edgesCover(E, A, B, (px << kSubpixelLog2) + sampleOffsetX(S, i), (py << kSubpixelLog2) + sampleOffsetY(S, i)))
            m |= 1u << i;
    return m;
}

// Depth of sample i of pixel (X, Y) (FineRaster.inl:695, 1047, 1096).
template <int S>
__device__ __forceinline__ U32 sampleDepth(U32 zx, U32 zy, U32 zb, U32 X, U32 Y, int i) {
    if (S == 0) return zx * X + zy * Y + zb;
    return zx * (U32)msaaPatternX(S, i) + zy * (U32)i + (((zx * X + zy * Y) << S) + zb);
}

// Pixel box [bx0, bx1] x [by0, by1] of the tile that can hold covered samples.
template <int S>
__device__ __forceinline__ bool pixelBox(const TileEdges& t, S32& bx0, S32& bx1, S32& by0, S32& by1) {
    const S32 pad = (S == 0) ? 0 : 8;
    bx0 = max(0, (t.minX - pad + 15) >> kSubpixelLog2);
    bx1 = min(7, (t.maxX + pad) >> kSubpixelLog2);
    by0 = max(0, (t.minY - pad + 15) >> kSubpixelLog2);
    by1 = min(7, (t.maxY + pad) >> kSubpixelLog2);
    return bx0 <= bx1 && by0 <= by1;
}

// Runs the fragment shader of triangle data td (16 words) at pixel (X, Y).
template <class FS, int S, U32 F>
__device__ __forceinline__ U32 shadeFragment(const U32* td, S32 triIdx, S32 X, S32 Y, U32 sampleMask,
                                             const float4* verts, S32 stride4, volatile F32* shared, U32 laneMask,
                                             bool& discard) {
    FS fs;
    fs.m_triIdx = triIdx;
    fs.m_vertIdx = FW::Vec3i((S32)td[13], (S32)td[14], (S32)td[15]);
    fs.m_pixelPos = FW::Vec2i(X, Y);
    fs.m_vertexBytes = stride4 * 16;
    fs.m_shared = shared;
    fs.m_vertices = verts;
    fs.m_laneMask = laneMask;
    fs.m_color = 0xFF0000FFu;
    fs.m_discard = false;
    if (!(F & kRenderLerp)) {
        // Interpolation disabled => varyings at the last vertex (FineRaster.inl:71-81).
        fs.m_center = FW::Vec3f(0.0f, 0.0f, 1.0f);
        fs.m_centerDX = FW::Vec3f(0.0f);
        fs.m_centerDY = FW::Vec3f(0.0f);
        fs.m_centroid = fs.m_center;
        fs.m_centroidDX = fs.m_centerDX;
        fs.m_centroidDY = fs.m_centerDY;
    } else {
        using Reads = FW::FragmentShaderReads<FS>;
        if (Reads::center || (S == 0 && Reads::centroid))
            computeBarys<S>(fs.m_center, fs.m_centerDX, fs.m_centerDY, td + 4, td + 7, td + 10, (X * 2 + 1) << S,
                            (Y * 2 + 1) << S);
        if (S == 0) {
            fs.m_centroid = fs.m_center;
            fs.m_centroidDX = fs.m_centerDX;
            fs.m_centroidDY = fs.m_centerDY;
        } else if (Reads::centroid) {
            U32 c = centroidCode(S, sampleMask);
            computeBarys<S>(fs.m_centroid, fs.m_centroidDX, fs.m_centroidDY, td + 4, td + 7, td + 10,
                            (X << (S + 1)) + (S32)(c & 0xF), (Y << (S + 1)) + (S32)(c >> 4));
        }
    }
    fs.run();
    discard = fs.m_discard;
    return fs.m_color;
}

template <class V, class FS, class BS, int S, U32 F>
__device__ __forceinline__ void fineTiles(const DrawDev& d, int group, S32 tileBegin, S32 tileEnd) {
    constexpr int NS = 1 << S;
    constexpr int TW = 64 << S;
    using Traits = FineTraits<FS, BS, S, F>;
    constexpr bool kDepth = Traits::kDepth;
    constexpr bool kQuads = Traits::kQuads;
    constexpr bool kVisibility = Traits::kVisibility;
    extern __shared__ __align__(16) unsigned char fineSmemRaw[];
    typename Traits::Smem& sm = reinterpret_cast<typename Traits::Smem*>(fineSmemRaw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const U32 ltMask = (1u << lane) - 1u;
    pdlWait();
    pdlTrigger();
    if (d.hostCounters != nullptr && blockIdx.x == 0 && threadIdx.x < (int)(sizeof(Counters) / 4))
        reinterpret_cast<volatile U32*>(d.hostCounters)[threadIdx.x] =
            reinterpret_cast<const volatile U32*>(d.counters)[threadIdx.x];
    if (__ldg(&d.counters->overflow)) return;
    const S32 selfPixels = d.fineSelfPixels > 0 ? d.fineSelfPixels : fineSelfPixelsDefault(S, kVisibility);

    // A warp's tiles come from the counter in increasing order: its current
    // instance stays valid until a tile reaches the next instance's first.
    int ii = 0;
    S32 instEnd = -1;
    for (;;) {
        S32 tile = 0;
        if (lane == 0) tile = atomicAdd(&d.fineTileCounter[group], 1);
        tile = __shfl_sync(0xFFFFFFFFu, tile, 0) + tileBegin;
        if (tile >= tileEnd) break;

        if (tile >= instEnd) {
            ii = findInstance(d.tilePrefix, d.numInstances, tile);
            instEnd = __ldg(&d.tilePrefix[ii + 1]);   // the prefix has numInstances + 1 entries
        }
        const InstanceDev* in = &d.inst[ii];
        const S32 wt = __ldg(&in->widthTiles);
        const S32 lt = tile - __ldg(&in->tileBase);
        const S32 tx = lt % wt, ty = lt / wt;
        const S32 count = __ldg(&d.tileCount[tile]);
        const S32 start = __ldg(&d.tileStart[tile]);
        const bool clear = __ldg(&in->deferredClear) != 0;
        if (count == 0 && !clear) continue;

        const S32 width = __ldg(&in->width), height = __ldg(&in->height);
        const S64 rowWords = __ldg(&in->rowWords);
        U32* gColor = (U32*)__ldg((const unsigned long long*)&in->color);
        U32* gDepth = (U32*)__ldg((const unsigned long long*)&in->depth);
        const S64 tileOrigin = (S64)(ty * 8) * rowWords + (S64)tx * 8 * NS;

        // Load or clear the tile (FineRaster.inl:562-580, 916-934), and its
        // maximum depth for early Z.
        U32 tileZMax = 0;
        if constexpr (kVisibility) {
            // Visibility keys start as depth << 32 (no fragment yet).
            U32 z = 0;
            if (clear) {
                const U32 cc = __ldg(&in->clearColor), cd = __ldg(&in->clearDepth);
                for (int w = lane; w < TW; w += 32) { sm.color[w] = cc; sm.key[w] = (U64)cd << 32; }
                z = cd;
            } else {
                for (int w = lane; w < TW; w += 32) {
                    S64 g = tileOrigin + (S64)(w / (8 * NS)) * rowWords + (w % (8 * NS));
                    sm.color[w] = gColor[g];
                    const U32 dz = gDepth[g];
                    sm.key[w] = (U64)dz << 32;
                    z = max(z, dz);
                }
            }
            tileZMax = __reduce_max_sync(0xFFFFFFFFu, z);
            __syncwarp();
        } else {
            if (clear) {
                const U32 cc = __ldg(&in->clearColor), cd = __ldg(&in->clearDepth);
                for (int w = lane; w < TW; w += 32) { sm.color[w] = cc; sm.depth[w] = cd; }
            } else {
                for (int w = lane; w < TW; w += 32) {
                    S64 g = tileOrigin + (S64)(w / (8 * NS)) * rowWords + (w % (8 * NS));
                    sm.color[w] = gColor[g];
                    sm.depth[w] = gDepth[g];
                }
            }
            __syncwarp();
            if (kDepth) {
                U32 z = 0;
                for (int w = lane; w < TW; w += 32) z = max(z, sm.depth[w]);
                tileZMax = __reduce_max_sync(0xFFFFFFFFu, z);
            }
        }

        // Pixel (0, 0) centre of the tile in the header frame.
        const S32 cx0 = ((tx * 8) << kSubpixelLog2) - ((width - 1) << (kSubpixelLog2 - 1));
        const S32 cy0 = ((ty * 8) << kSubpixelLog2) - ((height - 1) << (kSubpixelLog2 - 1));
        const S64 triBase = __ldg(&in->triBase);
        const S32 stride4 = __ldg(&in->stride4);
        const float4* verts = (const float4*)__ldg((const unsigned long long*)&in->vertices);

        // Visibility keys: depth << 32 | order, order = list position + 1; with
        // MSAA the low word also carries the winner's coverage mask of the
        // pixel (order << 8 | mask) while positions fit in 24 bits.
        const bool packed = S != 0 && count < (1 << 24) - 1;

        for (S32 batch = 0; batch < count; batch += 32) {
            if constexpr (kVisibility) {
                // ---- Visibility. Every (triangle, pixel) pair of the batch's
                // triangles whose pixel box has at most selfPixels pixels is
                // dealt to the lanes in turn, 32 pairs a pass: pair p's
                // triangle is the last one whose pairs start at or before p
                // (one OR over the warp marks the pass's starts, the
                // triangle of the previous pass's last pair carries over),
                // its pixel follows by an exact multiply-shift division by
                // the box width (a lane walking its own triangle's box
                // measured slower, even for boxes of one or two pixels);
                // larger triangles are rasterized by the whole warp, two
                // pixels per lane. Keys resolve by atomic minimum, so the
                // order pairs are taken in does not change a bit.
                S32 n = 0;
                bool big = false;
                if (batch + lane < count) {
                    const U32 entry = __ldg(&d.tileList[start + batch + lane]);
                    const U32 tri = entry >> 3, sub = entry & 7;
                    const S64 slot = (sub == 7) ? (S64)tri : (S64)__ldg(&d.triHeader[tri].w) + sub;
                    const uint4 h = __ldg(&d.triHeader[slot]);
                    if ((h.w & 0xFFFFF000u) < tileZMax) {
                        const TileEdges te = tileEdges(h, cx0, cy0);
                        S32 bx0, bx1, by0, by1;
                        if (pixelBox<S>(te, bx0, bx1, by0, by1)) {
                            const uint4 q0 = __ldg(&d.triData[slot * 4]);
                            const S32 w = bx1 - bx0 + 1;
                            const S32 cnt = w * (by1 - by0 + 1);
                            big = cnt > selfPixels;
                            sm.rec[lane].q[0] = make_uint4((U32)te.E[0], (U32)te.E[1], (U32)te.E[2], (U32)te.A[0]);
                            sm.rec[lane].q[1] = make_uint4((U32)te.A[1], (U32)te.A[2], (U32)te.B[0], (U32)te.B[1]);
                            sm.rec[lane].q[2] = make_uint4((U32)te.B[2], q0.x, q0.y, q0.z);
                            if (!big) {
                                n = cnt;
                                // Row of box pixel k: (k * ceil(2^16 / w)) >> 16, exact for k < 64, w <= 8.
                                sm.box[lane] = (U32)bx0 | (U32)by0 << 4 | (U32)w << 8 |
                                               ((65536u + (U32)w - 1u) / (U32)w) << 12;
                            }
                        }
                    }
                }
                S32 P = 0, myStart = 0;
                if (__any_sync(0xFFFFFFFFu, n > 0)) {
                    S32 incl = n;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const S32 t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                        if (lane >= o) incl += t;
                    }
                    myStart = incl - n;
                    P = __shfl_sync(0xFFFFFFFFu, incl, 31);
                }
                __syncwarp();
                S32 carryJ = 0, carryStart = 0;   // triangle (and its first pair) of the last pair so far
                for (S32 base = 0; base < P; base += 32) {
                    const bool starts = n > 0 && myStart >= base && myStart < base + 32;
                    if (starts) sm.head[myStart - base] = lane;
                    const U32 startMask = __reduce_or_sync(0xFFFFFFFFu, starts ? 1u << (myStart - base) : 0u);
                    __syncwarp();
                    const U32 upTo = startMask & (0xFFFFFFFFu >> (31 - lane));
                    S32 j = carryJ, first = carryStart;
                    if (upTo) {
                        const int h = 31 - __clz(upTo);
                        j = sm.head[h];
                        first = base + h;
                    }
                    carryJ = __shfl_sync(0xFFFFFFFFu, j, 31);
                    carryStart = __shfl_sync(0xFFFFFFFFu, first, 31);
                    __syncwarp();   // every lane has read head before the next pass rewrites it
                    const S32 p = base + lane;
                    if (p >= P) continue;
                    const S32 k = p - first;
                    const U32 bw = sm.box[j];
                    const S32 w = (S32)((bw >> 8) & 0xFu);
                    const S32 q = (S32)(((U32)k * (bw >> 12)) >> 16);
                    const S32 px = (S32)(bw & 0xFu) + k - q * w, py = (S32)((bw >> 4) & 0xFu) + q;
                    const uint4 r0 = sm.rec[j].q[0], r1 = sm.rec[j].q[1], r2 = sm.rec[j].q[2];
                    const S32 E[3] = {(S32)r0.x, (S32)r0.y, (S32)r0.z};
                    const S32 A[3] = {(S32)r0.w, (S32)r1.x, (S32)r1.y};
                    const S32 B[3] = {(S32)r1.z, (S32)r1.w, (S32)r2.x};
                    const U32 smask = sampleMaskOf<S>(E, A, B, px, py);
                    if (!smask) continue;
                    const U32 order = (U32)(batch + j + 1);
                    const U64 low = packed ? (order << 8 | smask) : order;
                    const U32 X = (U32)(tx * 8 + px), Y = (U32)(ty * 8 + py);
                    const U32 zx = r2.y, zy = r2.z, zb = r2.w;
#pragma unroll
                    for (int i = 0; i < NS; i++) {
                        if (!(smask >> i & 1)) continue;
                        const int idx = py * 8 * NS + i * 8 + px;
                        const U64 key = ((U64)sampleDepth<S>(zx, zy, zb, X, Y, i) << 32) | low;
                        if (key < sm.key[idx]) atomicMin((unsigned long long*)&sm.key[idx], (unsigned long long)key);
                    }
                }
                __syncwarp();
                // Larger triangles: the whole warp, one at a time, in batch
                // order (each lane owns its two pixels, so plain stores
                // suffice). At one sample a lane keeps its two keys in
                // registers over all of them: the row below is 4 pixels
                // (64 subpixels) down, so its edge values are the first
                // row's plus 64 B and its depth the first's plus 4 zy; a
                // sample is covered iff no edge value is negative, i.e. iff
                // their OR is not.
                const S32 px = lane & 7, py0 = lane >> 3, py1 = py0 + 4;
                const U32 pX = (U32)(tx * 8 + px), pY0 = (U32)(ty * 8 + py0), pY1 = pY0 + 4;
                U32 bigMask = __ballot_sync(0xFFFFFFFFu, big);
                if (S == 0 && bigMask) {
                    const int idx0 = py0 * 8 + px, idx1 = idx0 + 32;
                    U64 k0 = sm.key[idx0], k1 = sm.key[idx1];
                    const S32 qx = px << kSubpixelLog2, qy = py0 << kSubpixelLog2;
                    for (; bigMask; bigMask &= bigMask - 1) {
                        const int j = __ffs(bigMask) - 1;
                        const uint4 r0 = sm.rec[j].q[0], r1 = sm.rec[j].q[1], r2 = sm.rec[j].q[2];
                        const S32 e00 = (S32)r0.x + (S32)r0.w * qx + (S32)r1.z * qy;
                        const S32 e01 = (S32)r0.y + (S32)r1.x * qx + (S32)r1.w * qy;
                        const S32 e02 = (S32)r0.z + (S32)r1.y * qx + (S32)r2.x * qy;
                        const S32 e10 = e00 + ((S32)r1.z << (kSubpixelLog2 + 2));
                        const S32 e11 = e01 + ((S32)r1.w << (kSubpixelLog2 + 2));
                        const S32 e12 = e02 + ((S32)r2.x << (kSubpixelLog2 + 2));
                        const U32 z0 = r2.y * pX + r2.z * pY0 + r2.w, z1 = z0 + (r2.z << 2);
                        const U32 order = (U32)(batch + j + 1);
                        const U64 key0 = ((U64)z0 << 32) | order, key1 = ((U64)z1 << 32) | order;
                        if ((e00 | e01 | e02) >= 0 && key0 < k0) k0 = key0;
                        if ((e10 | e11 | e12) >= 0 && key1 < k1) k1 = key1;
                    }
                    sm.key[idx0] = k0;
                    sm.key[idx1] = k1;
                }
                for (; bigMask; bigMask &= bigMask - 1) {
                    const int j = __ffs(bigMask) - 1;
                    const uint4 r0 = sm.rec[j].q[0], r1 = sm.rec[j].q[1], r2 = sm.rec[j].q[2];
                    const S32 E[3] = {(S32)r0.x, (S32)r0.y, (S32)r0.z};
                    const S32 A[3] = {(S32)r0.w, (S32)r1.x, (S32)r1.y};
                    const S32 B[3] = {(S32)r1.z, (S32)r1.w, (S32)r2.x};
                    const U32 zx = r2.y, zy = r2.z, zb = r2.w;
                    const U32 order = (U32)(batch + j + 1);
#pragma unroll
                    for (int half = 0; half < 2; half++) {
                        const S32 pyy = half ? py1 : py0;
                        const U32 Y = half ? pY1 : pY0;
                        const U32 smask = sampleMaskOf<S>(E, A, B, px, pyy);
                        const U64 low = packed ? (order << 8 | smask) : order;
#pragma unroll
                        for (int i = 0; i < NS; i++) {
                            if (!(smask >> i & 1)) continue;
                            const int idx = pyy * 8 * NS + i * 8 + px;
                            const U64 key = ((U64)sampleDepth<S>(zx, zy, zb, pX, Y, i) << 32) | low;
                            if (key < sm.key[idx]) sm.key[idx] = key;
                        }
                    }
                }
                __syncwarp();
                // Exact current depth maximum for the next batch's early Z.
                U32 z = 0;
                for (int w = lane; w < TW; w += 32) z = max(z, (U32)(sm.key[w] >> 32));
                tileZMax = __reduce_max_sync(0xFFFFFFFFu, z);
            } else {
                // ---- 1. One triangle per lane: its words in shared memory, and
                // the pixels of the small ones (box of at most selfPixels pixels)
                // as (triangle, pixel) pairs dealt over the lanes, each setting
                // the triangle's coverage bit of its pixel (the masks do not
                // depend on the order the pairs are taken in).
                bool valid = batch + lane < count;
                bool self = false;     // small triangle: covered through the pairs
                U32 myLo = 0, myHi = 0;
                S32 n = 0;
                U32* pairBox = sm.pairBox;
                U32* pairMul = sm.pairMul;
                sm.covLo[lane] = 0u;
                sm.covHi[lane] = 0u;
                // Batch filter (see step 2b): exact for single-sample depth-tested
                // pipes whose fragment shader never discards.
                constexpr bool kFilter = S == 0 && kDepth && !kQuads && !FW::FragmentShaderTraits<FS>::mayDiscard;
                if constexpr (kFilter) {
                    sm.batchMin[lane] = ~0ull;
                    sm.batchMin[lane + 32] = ~0ull;
                }
                if (valid) {
                    U32 entry = __ldg(&d.tileList[start + batch + lane]);
                    U32 tri = entry >> 3, sub = entry & 7;
                    S64 slot = (sub == 7) ? (S64)tri : (S64)__ldg(&d.triHeader[tri].w) + sub;
                    uint4 h = __ldg(&d.triHeader[slot]);
                    if (kDepth && (h.w & 0xFFFFF000u) >= tileZMax) valid = false;
                    if (valid) {
                        const TileEdges te = tileEdges(h, cx0, cy0);
                        const uint4* tdp = &d.triData[slot * 4];
                        uint4 q0 = __ldg(&tdp[0]);
                        S32 bx0, bx1, by0, by1;
                        const bool inTile = pixelBox<S>(te, bx0, bx1, by0, by1);
                        const S32 w = bx1 - bx0 + 1;
                        self = !inTile || w * (by1 - by0 + 1) <= selfPixels;
#pragma unroll
                        for (int k = 0; k < 3; k++) {
                            sm.E[k][lane] = te.E[k];
                            sm.A[k][lane] = te.A[k];
                            sm.B[k][lane] = te.B[k];
                        }
                        sm.td[0][lane] = q0.x; sm.td[1][lane] = q0.y; sm.td[2][lane] = q0.z; sm.td[3][lane] = q0.w;
                        uint4 q1 = __ldg(&tdp[1]), q2 = __ldg(&tdp[2]), q3 = __ldg(&tdp[3]);
                        sm.td[4][lane] = q1.x; sm.td[5][lane] = q1.y; sm.td[6][lane] = q1.z; sm.td[7][lane] = q1.w;
                        sm.td[8][lane] = q2.x; sm.td[9][lane] = q2.y; sm.td[10][lane] = q2.z; sm.td[11][lane] = q2.w;
                        sm.td[12][lane] = q3.x; sm.td[13][lane] = q3.y; sm.td[14][lane] = q3.z; sm.td[15][lane] = q3.w;
                        sm.tri[lane] = (S32)((S64)tri - triBase);
                        // No pixel of the tile can be covered (!inTile): nothing to do.
                        if (inTile && self) {
                            n = w * (by1 - by0 + 1);
                            pairBox[lane] = (U32)bx0 | (U32)by0 << 4 | (U32)w << 8;
                            // Row of box pixel k: (k * ceil(2^16 / w)) >> 16, exact for k < 64, w <= 8.
                            pairMul[lane] = (65536u + (U32)w - 1u) / (U32)w;
                        }
                    }
                }
                S32 P = 0;
                if (__any_sync(0xFFFFFFFFu, n > 0)) {
                    S32 incl = n;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const S32 t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                        if (lane >= o) incl += t;
                    }
                    sm.fragEnd[lane] = incl;
                    P = __shfl_sync(0xFFFFFFFFu, incl, 31);
                }
                __syncwarp();
                for (S32 base = 0; base < P; base += 32) {
                    const S32 p = base + lane;
                    if (p >= P) continue;
                    int j = 0;
#pragma unroll
                    for (int s2 = 16; s2 > 0; s2 >>= 1)
                        if (sm.fragEnd[j + s2 - 1] <= p) j += s2;
                    const S32 k = p - (j ? sm.fragEnd[j - 1] : 0);
                    const U32 bw = pairBox[j];
                    const S32 w = (S32)(bw >> 8);
                    const S32 q = (S32)(((U32)k * pairMul[j]) >> 16);
                    const S32 px = (S32)(bw & 0xFu) + k - q * w, py = (S32)((bw >> 4) & 0xFu) + q;
                    const S32 qx = px << kSubpixelLog2, qy = py << kSubpixelLog2;
                    bool c = true;
#pragma unroll
                    for (int e = 0; e < 3; e++) {
                        const S32 a = sm.A[e][j], b = sm.B[e][j];
                        const S32 slack = (S == 0) ? 0 : (abs(a) + abs(b)) << (kSubpixelLog2 - 1);
                        c = c && (sm.E[e][j] + a * qx + b * qy + slack >= 0);
                    }
                    if (kDepth && S == 0 && !kQuads && c) {
                        const U32 X = (U32)(tx * 8 + px), Y = (U32)(ty * 8 + py);
                        const U32 z = sm.td[0][j] * X + sm.td[1][j] * Y + sm.td[2][j];
                        c = z < sm.depth[py * 8 + px];
                        if constexpr (kFilter)
                            if (c) atomicMin((unsigned long long*)&sm.batchMin[py * 8 + px], ((unsigned long long)z << 32) | (U32)j);
                    }
                    if (c) {
                        const int bit = py * 8 + px;
                        atomicOr(bit < 32 ? &sm.covLo[j] : &sm.covHi[j], 1u << (bit & 31));
                    }
                }
                __syncwarp();
                if (self) {
                    myLo = sm.covLo[lane];
                    myHi = sm.covHi[lane];
                }
                U64 min0 = 0, min1 = 0;   // batch minima of this lane's pixels (lane, lane + 32)
                if constexpr (kFilter) {
                    min0 = sm.batchMin[lane];
                    min1 = sm.batchMin[lane + 32];
                }
                __syncwarp();
                const U32 coopMask = __ballot_sync(0xFFFFFFFFu, valid && !self);

                // ---- 2. Large triangles, two pixels per lane.
                const S32 px = lane & 7, py0 = lane >> 3, py1 = py0 + 4;
                const U32 pX = (U32)(tx * 8 + px), pY0 = (U32)(ty * 8 + py0);
                {
                    // Single-sample depth of this lane's two pixels at the start of
                    // the batch: a fragment that fails against it fails in
                    // submission order too (depths only decrease).
                    U32 curZ0 = 0, curZ1 = 0;
                    if (kDepth && S == 0 && !kQuads) {
                        curZ0 = sm.depth[lane];
                        curZ1 = sm.depth[lane + 32];
                    }
                    const S32 qx = px << kSubpixelLog2, qy0 = py0 << kSubpixelLog2, qy1 = py1 << kSubpixelLog2;
                    for (U32 m = coopMask; m; m &= m - 1) {
                        const int j = __ffs(m) - 1;
                        bool c0 = true, c1 = true;
#pragma unroll
                        for (int k = 0; k < 3; k++) {
                            S32 e = sm.E[k][j], a = sm.A[k][j], b = sm.B[k][j];
                            S32 base = e + a * qx;
                            S32 slack = (S == 0) ? 0 : (abs(a) + abs(b)) << (kSubpixelLog2 - 1);
                            c0 = c0 && (base + b * qy0 + slack >= 0);
                            c1 = c1 && (base + b * qy1 + slack >= 0);
                        }
                        if (kDepth && S == 0 && !kQuads) {
                            const U32 zx = sm.td[0][j], zy = sm.td[1][j], zb = sm.td[2][j];
                            const U32 z0 = zx * pX + zy * pY0 + zb, z1 = z0 + zy * 4u;
                            c0 = c0 && (z0 < curZ0);
                            c1 = c1 && (z1 < curZ1);
                            if constexpr (kFilter) {
                                const U64 k0 = ((U64)z0 << 32) | (U32)j, k1 = ((U64)z1 << 32) | (U32)j;
                                if (c0 && k0 < min0) min0 = k0;
                                if (c1 && k1 < min1) min1 = k1;
                            }
                        }
                        U32 lo = __ballot_sync(0xFFFFFFFFu, c0);
                        U32 hi = __ballot_sync(0xFFFFFFFFu, c1);
                        if (lane == j) { myLo = lo; myHi = hi; }
                    }
                }
                if (kQuads) {
                    // quadCoverage (FineRaster.inl:401-406): bit of the quad's top-left pixel.
                    U64 c = ((U64)myHi << 32) | myLo;
                    c |= c >> 1;
                    c |= c >> 8;
                    c &= 0x0055005500550055ull;
                    myLo = (U32)c;
                    myHi = (U32)(c >> 32);
                }
                if constexpr (kFilter) {
                    // ---- 2b. A fragment of pixel p later in the batch than p's
                    // minimum (depth, then batch position) fails the in-order LESS
                    // test: the minimum's own fragment passes (every earlier one is
                    // deeper) and leaves the depth at or below the later one's, and
                    // without discard nothing else changes it. Triangle j keeps
                    // the pixels whose minimum is at j or later: a bit-sliced
                    // comparison of the 5-bit positions (10 ballots) against j.
                    const U32 w0 = min((U32)min0, 31u), w1 = min((U32)min1, 31u);
                    U32 gtLo = 0u, eqLo = ~0u, gtHi = 0u, eqHi = ~0u;
#pragma unroll
                    for (int b = 4; b >= 0; b--) {
                        const U32 pl = __ballot_sync(0xFFFFFFFFu, (w0 >> b) & 1u);
                        const U32 ph = __ballot_sync(0xFFFFFFFFu, (w1 >> b) & 1u);
                        const U32 jb = 0u - (((U32)lane >> b) & 1u);   // bit b of this lane's triangle j
                        gtLo |= eqLo & pl & ~jb;
                        eqLo &= ~(pl ^ jb);
                        gtHi |= eqHi & ph & ~jb;
                        eqHi &= ~(ph ^ jb);
                    }
                    myLo &= gtLo | eqLo;
                    myHi &= gtHi | eqHi;
                }
                if (!valid) { myLo = 0; myHi = 0; }

                // ---- 3. Fragment compaction in submission order.
                const S32 pop = (__popc(myLo) + __popc(myHi)) * (kQuads ? 4 : 1);
                S32 inc = pop;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    S32 t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                    if (lane >= o) inc += t;
                }
                const S32 myFragStart = inc - pop;
                S32 fragCarryJ = 0, fragCarryStart = 0;   // triangle (and its first fragment) of the last fragment so far
                sm.covLo[lane] = myLo;
                sm.covHi[lane] = myHi;
                const S32 total = __shfl_sync(0xFFFFFFFFu, inc, 31);
                __syncwarp();

                for (S32 pass = 0; pass < total; pass += 32) {
                    const S32 f = pass + lane;
                    bool act = f < total;
                    int j = 0, pixel = 0;
                    bool covered = false;
                    U32 sampleMask = 0;
                    U32 dz[NS];
                    // Triangle of fragment f: the last one whose fragments start
                    // at or before f (one OR over the warp marks the pass's
                    // starts; the triangle of the previous pass's last fragment
                    // carries over).
                    const bool startsHere = pop > 0 && myFragStart >= pass && myFragStart < pass + 32;
                    if (startsHere) sm.fragHead[myFragStart - pass] = lane;
                    const U32 startMask = __reduce_or_sync(0xFFFFFFFFu, startsHere ? 1u << (myFragStart - pass) : 0u);
                    __syncwarp();
                    const U32 upTo = startMask & (0xFFFFFFFFu >> (31 - lane));
                    int fragJ = fragCarryJ;
                    S32 fragFirst = fragCarryStart;
                    if (upTo) {
                        const int h = 31 - __clz(upTo);
                        fragJ = sm.fragHead[h];
                        fragFirst = pass + h;
                    }
                    fragCarryJ = __shfl_sync(0xFFFFFFFFu, fragJ, 31);
                    fragCarryStart = __shfl_sync(0xFFFFFFFFu, fragFirst, 31);
                    __syncwarp();   // every lane has read fragHead before the next pass rewrites it
                    if (act) {
                        j = fragJ;
                        const U32 cl = sm.covLo[j], ch = sm.covHi[j];
                        const S32 k = f - fragFirst;
                        if (kQuads) {
                            int qbit = nthSetBit64(cl, ch, k >> 2);
                            pixel = qbit + (k & 1) + ((k & 2) << 2);  // findFragment, FineRaster.inl:417-427
                        } else {
                            pixel = nthSetBit64(cl, ch, k);
                        }
                        const S32 fx = pixel & 7, fy = pixel >> 3;
                        if (S == 0 && !kQuads) {
                            sampleMask = 1;  // single-sample masks are exact
                        } else {
                            const S32 E[3] = {sm.E[0][j], sm.E[1][j], sm.E[2][j]};
                            const S32 A[3] = {sm.A[0][j], sm.A[1][j], sm.A[2][j]};
                            const S32 B[3] = {sm.B[0][j], sm.B[1][j], sm.B[2][j]};
                            sampleMask = sampleMaskOf<S>(E, A, B, fx, fy);
                        }
                        covered = sampleMask != 0;
                        if (!kQuads && !covered) act = false;
                        const U32 X = (U32)(tx * 8 + fx), Y = (U32)(ty * 8 + fy);
                        if (kDepth) {
                            const U32 zx = sm.td[0][j], zy = sm.td[1][j], zb = sm.td[2][j];
                            bool anyPass = false;
                            const int rowBase = fy * 8 * NS + fx;
#pragma unroll
                            for (int i = 0; i < NS; i++) {
                                dz[i] = sampleDepth<S>(zx, zy, zb, X, Y, i);
                                if ((sampleMask >> i & 1) && dz[i] < sm.depth[rowBase + i * 8]) anyPass = true;
                            }
                            if (!kQuads && !anyPass) act = false;
                            if (kQuads && !anyPass) covered = false;
                        }
                    }
                    // Shade.
                    const U32 shadeMask = __ballot_sync(0xFFFFFFFFu, act);
                    U32 src = 0;
                    bool discard = true;
                    if (act) {
                        U32 td[16];
#pragma unroll
                        for (int q = 0; q < 16; q++) td[q] = sm.td[q][j];
                        src = shadeFragment<FS, S, F>(td, sm.tri[j], tx * 8 + (pixel & 7), ty * 8 + (pixel >> 3), sampleMask,
                                                      verts, stride4, sm.shared, shadeMask, discard);
                    }
                    // ROP: same-pixel fragments of this pass applied in lane order.
                    const bool rop = act && covered && !discard;
                    const U32 ropMask = __ballot_sync(0xFFFFFFFFu, rop);
                    if (ropMask) {
                        U32 peers = 0;
                        if (rop) peers = __match_any_sync(ropMask, pixel);
                        const int rank = __popc(peers & ltMask);
                        const int maxGroup = __reduce_max_sync(0xFFFFFFFFu, rop ? __popc(peers) : 0);
                        for (int r = 0; r < maxGroup; r++) {
                            if (rop && rank == r) {
                                const S32 fx = pixel & 7, fy = pixel >> 3;
                                const int rowBase = fy * 8 * NS + fx;
                                BS bs;
#pragma unroll
                                for (int i = 0; i < NS; i++) {
                                    if (!(sampleMask >> i & 1)) continue;
                                    const int idx = rowBase + i * 8;
                                    if (kDepth) {
                                        if (!(dz[i] < sm.depth[idx])) continue;
                                        sm.depth[idx] = dz[i];
                                    }
                                    bs.m_triIdx = sm.tri[j];
                                    bs.m_pixelPos = FW::Vec2i(tx * 8 + fx, ty * 8 + fy);
                                    bs.m_sampleIdx = i;
                                    bs.m_src = src;
                                    bs.m_dst = sm.color[idx];
                                    bs.m_color = 0xFF0000FFu;
                                    bs.m_writeColor = true;
                                    bs.run();
                                    if (bs.m_writeColor) sm.color[idx] = bs.m_color;
                                }
                            }
                            __syncwarp();
                        }
                    }
                }
                if (kDepth) {
                    U32 z = 0;
                    for (int w = lane; w < TW; w += 32) z = max(z, sm.depth[w]);
                    tileZMax = __reduce_max_sync(0xFFFFFFFFu, z);
                }
                __syncwarp();
            }
        }

        if constexpr (kVisibility) {
            // ---- Resolve: shade every (pixel, winning triangle) once. Sample
            // i0 of a pixel starts a winner if no earlier sample of the pixel
            // has the same key low word (with MSAA the low word carries the
            // winner's coverage mask, so neither its edges nor its mask are
            // recomputed here). The winners of the tile are listed first (a
            // lane owns pixels lane and lane + 32), then fetched and shaded
            // 32 at a time, so lanes stay busy however unevenly the winners
            // fall on the pixels and samples.
            U32* winners = sm.winners;
            S32 nw = 0;
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int p = lane + 32 * hh;
                const int rowBase = (p >> 3) * 8 * NS + (p & 7);
                U32 mine[NS];
                int cnt = 0;
#pragma unroll
                for (int i0 = 0; i0 < NS; i0++) {
                    const U32 low = (U32)sm.key[rowBase + i0 * 8];
                    bool first = low != 0;
#pragma unroll
                    for (int i = 0; i < i0; i++)
                        if ((U32)sm.key[rowBase + i * 8] == low) first = false;
                    U32 won = 0;
                    if (first) {
#pragma unroll
                        for (int i = 0; i < NS; i++)
                            if ((U32)sm.key[rowBase + i * 8] == low) won |= 1u << i;
                    }
                    mine[i0] = (U32)p | (U32)i0 << 6 | won << 9;
                    cnt += first ? 1 : 0;
                }
                S32 pos = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const S32 t = __shfl_up_sync(0xFFFFFFFFu, pos, o);
                    if (lane >= o) pos += t;
                }
                const S32 total = __shfl_sync(0xFFFFFFFFu, pos, 31);
                pos += nw - cnt;
#pragma unroll
                for (int i0 = 0; i0 < NS; i0++)
                    if (mine[i0] >> 9) winners[pos++] = mine[i0];
                nw += total;
            }
            __syncwarp();
            for (S32 w0 = 0; w0 < nw; w0 += 32) {
                if (w0 + lane >= nw) continue;
                const U32 rec = winners[w0 + lane];
                const int p = (int)(rec & 63u), i0 = (int)((rec >> 6) & 7u);
                const U32 won = rec >> 9;
                const S32 px = p & 7, py = p >> 3;
                const int rowBase = py * 8 * NS + px;
                U32 low = (U32)sm.key[rowBase + i0 * 8];
                U32 td[16];
                const U32 entry = __ldg(&d.tileList[start + (S32)(packed ? (low >> 8) : low) - 1]);
                const U32 sub = entry & 7;
                const U32 tri = entry >> 3;
                const S64 slot = (sub == 7) ? (S64)tri : (S64)__ldg(&d.triHeader[tri].w) + sub;
                const uint4* tdp = &d.triData[slot * 4];
                const uint4 q1 = __ldg(&tdp[1]), q2 = __ldg(&tdp[2]), q3 = __ldg(&tdp[3]);
                td[4] = q1.x; td[5] = q1.y; td[6] = q1.z; td[7] = q1.w;
                td[8] = q2.x; td[9] = q2.y; td[10] = q2.z; td[11] = q2.w;
                td[12] = q3.x; td[13] = q3.y; td[14] = q3.z; td[15] = q3.w;
                if (S != 0 && !packed) {
                    const TileEdges te = tileEdges(__ldg(&d.triHeader[slot]), cx0, cy0);
                    low = sampleMaskOf<S>(te.E, te.A, te.B, px, py);
                } else if (S != 0) {
                    low &= 0xFFu;
                }
                bool discard;
                const S32 X = tx * 8 + px, Y = ty * 8 + py;
                const S32 triIdx = (S32)((S64)tri - triBase);
                // low now holds the winner's coverage mask of the pixel (MSAA).
                const U32 src = shadeFragment<FS, S, F>(td, triIdx, X, Y, S != 0 ? low : 1u, verts, stride4,
                                                        sm.shared, 0u, discard);
                BS bs;
#pragma unroll
                for (int i = 0; i < NS; i++) {
                    if (!(won >> i & 1)) continue;
                    const int idx = rowBase + i * 8;
                    bs.m_triIdx = triIdx;
                    bs.m_pixelPos = FW::Vec2i(X, Y);
                    bs.m_sampleIdx = i;
                    bs.m_src = src;
                    bs.m_dst = sm.color[idx];
                    bs.m_color = 0xFF0000FFu;
                    bs.m_writeColor = true;
                    bs.run();
                    if (bs.m_writeColor) sm.color[idx] = bs.m_color;
                }
            }
            __syncwarp();
        }

        // Write the tile back (FineRaster.inl:736-746).
        for (int w = lane; w < TW; w += 32) {
            S64 g = tileOrigin + (S64)(w / (8 * NS)) * rowWords + (w % (8 * NS));
            gColor[g] = sm.color[w];
            if constexpr (kVisibility)
                gDepth[g] = (U32)(sm.key[w] >> 32);
            else
                gDepth[g] = sm.depth[w];
        }
        __syncwarp();
    }
}

// The fine-stage kernel. At one sample the register budget is pinned to five
// resident CTAs per SM (48 registers); with MSAA the compiler's own choice
// measured faster than any pinned budget (4x MSAA: 63 registers, 0.58 ms on
// the 4K grid, against 0.60 ms pinned to four CTAs, 0.64 ms to three and
// 0.645 ms to five, where 48 registers fit without spills but with more
// instructions).
template <class V, class FS, class BS, int S, U32 F>
__global__ void __launch_bounds__(kFineMaxThreads, 5) fineKernel1(DrawDev d, int group, S32 tileBegin, S32 tileEnd) {
    fineTiles<V, FS, BS, S, F>(d, group, tileBegin, tileEnd);
}
template <class V, class FS, class BS, int S, U32 F>
__global__ void __launch_bounds__(kFineMaxThreads) fineKernelMsaa(DrawDev d, int group, S32 tileBegin, S32 tileEnd) {
    fineTiles<V, FS, BS, S, F>(d, group, tileBegin, tileEnd);
}
template <class V, class FS, class BS, int S, U32 F>
constexpr auto fineKernelFor() {
    if constexpr (S == 0)
        return &fineKernel1<V, FS, BS, S, F>;
    else
        return &fineKernelMsaa<V, FS, BS, S, F>;
}

}  // namespace cr
