// fine.cuh -- fine raster kernel (stage 4 of 4).
//
// One warp owns one 8x8 tile at a time (persistent warps pulling tiles from a
// counter, as FineRaster.inl:534-552). The tile's colour and depth live in the
// warp's shared memory for the whole tile. Its triangle list is consumed in
// batches of 32:
//   1. lane i fetches entry i: header, data slot, early-Z against the tile's
//      current maximum depth (FineRaster.inl:229-240), edge functions at the
//      tile origin;
//   2. the 32 lanes, each owning two pixels, evaluate every triangle of the
//      batch and ballot a 64-bit pixel coverage mask per triangle;
//   3. covered pixels are compacted into passes of 32 fragments in
//      submission order (FineRaster.inl:625-731);
//   4. each fragment is depth-tested, shaded and blended. Fragments of the
//      same pass that hit the same pixel are grouped with __match_any_sync
//      and applied one rank at a time in lane order, which is submission
//      order. This replaces the reference's reliance on lock-step warps for
//      same-address shared-memory races (FineRaster.inl:433-495, 758-851),
//      which is undefined on sm_70 and later.
// MSAA keeps every sample of the tile in shared memory (reference layout:
// sample i of pixel x at word i * 8 + x of the tile row) and shades once per
// pixel at the centroid of the covered samples.
#pragma once

#include "../PixelPipe.hpp"
#include "device.cuh"

namespace cr {

template <int S>
struct FineWarpSmem {
    static constexpr int kTileWords = 64 << S;
    U32 color[kTileWords];
    U32 depth[kTileWords];
    S32 E[3][32];      // edge functions at the tile's pixel (0, 0) centre, bias folded in
    S32 A[3][32];      // per-subpixel x step (-dy)
    S32 B[3][32];      // per-subpixel y step (+dx)
    U32 td[16][32];    // triangle data slots (CRTriangleData words)
    S32 tri[32];       // triangle index within the draw
    U32 covLo[32];
    U32 covHi[32];
    S32 fragEnd[32];
    F32 shared[32];
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

constexpr int kFineMaxThreads = 256;

template <class V, class FS, class BS, int S, U32 F>
__global__ void __launch_bounds__(kFineMaxThreads) fineKernel(DrawDev d, int group, S32 tileBegin, S32 tileEnd) {
    constexpr int NS = 1 << S;
    constexpr int TW = 64 << S;
    constexpr bool kDepth = (F & kRenderDepth) != 0;
    constexpr bool kLerp = (F & kRenderLerp) != 0;
    constexpr bool kQuads = (F & kRenderQuads) != 0;
    extern __shared__ __align__(16) unsigned char fineSmemRaw[];
    FineWarpSmem<S>& sm = reinterpret_cast<FineWarpSmem<S>*>(fineSmemRaw)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const U32 ltMask = (1u << lane) - 1u;
    if (__ldg(&d.counters->overflow)) return;

    for (;;) {
        S32 tile = 0;
        if (lane == 0) tile = atomicAdd(&d.fineTileCounter[group], 1);
        tile = __shfl_sync(0xFFFFFFFFu, tile, 0) + tileBegin;
        if (tile >= tileEnd) break;

        const int ii = findInstance(d.tilePrefix, d.numInstances, tile);
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

        // Load or clear the tile (FineRaster.inl:562-580, 916-934).
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
        U32 tileZMax = 0;
        if (kDepth) {
            U32 z = 0;
            for (int w = lane; w < TW; w += 32) z = max(z, sm.depth[w]);
            tileZMax = __reduce_max_sync(0xFFFFFFFFu, z);
        }

        // Pixel (0, 0) centre of the tile in the header frame.
        const S32 cx0 = ((tx * 8) << kSubpixelLog2) - ((width - 1) << (kSubpixelLog2 - 1));
        const S32 cy0 = ((ty * 8) << kSubpixelLog2) - ((height - 1) << (kSubpixelLog2 - 1));
        const S64 triBase = __ldg(&in->triBase);
        const S32 stride4 = __ldg(&in->stride4);
        const float4* verts = (const float4*)__ldg((const unsigned long long*)&in->vertices);

        for (S32 batch = 0; batch < count; batch += 32) {
            // 1. Fetch one triangle per lane.
            bool valid = batch + lane < count;
            if (valid) {
                U32 entry = __ldg(&d.tileList[start + batch + lane]);
                U32 tri = entry >> 3, sub = entry & 7;
                S64 slot = (sub == 7) ? (S64)tri : (S64)__ldg(&d.triHeader[tri].w) + sub;
                uint4 h = __ldg(&d.triHeader[slot]);
                if (kDepth && (h.w & 0xFFFFF000u) >= tileZMax) valid = false;
                if (valid) {
                    S32 vx[3] = {lo16(h.x), lo16(h.y), lo16(h.z)};
                    S32 vy[3] = {hi16(h.x), hi16(h.y), hi16(h.z)};
                    // Edges (v0, v1 - v0), (v1, v2 - v1), (v0, v0 - v2) as FineRaster.inl:251-275.
                    const int oi[3] = {0, 1, 0};
                    S32 ddx[3] = {vx[1] - vx[0], vx[2] - vx[1], vx[0] - vx[2]};
                    S32 ddy[3] = {vy[1] - vy[0], vy[2] - vy[1], vy[0] - vy[2]};
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        S64 e = (S64)(vx[oi[k]] - cx0) * ddy[k] - (S64)(vy[oi[k]] - cy0) * ddx[k];
                        if (ddy[k] > 0 || (ddy[k] == 0 && ddx[k] <= 0)) e -= 1;  // Util.inl:100
                        sm.E[k][lane] = clampEdge(e);
                        sm.A[k][lane] = -ddy[k];
                        sm.B[k][lane] = ddx[k];
                    }
                    const uint4* td = &d.triData[slot * 4];
                    uint4 q0 = __ldg(&td[0]), q1 = __ldg(&td[1]), q2 = __ldg(&td[2]), q3 = __ldg(&td[3]);
                    sm.td[0][lane] = q0.x; sm.td[1][lane] = q0.y; sm.td[2][lane] = q0.z; sm.td[3][lane] = q0.w;
                    sm.td[4][lane] = q1.x; sm.td[5][lane] = q1.y; sm.td[6][lane] = q1.z; sm.td[7][lane] = q1.w;
                    sm.td[8][lane] = q2.x; sm.td[9][lane] = q2.y; sm.td[10][lane] = q2.z; sm.td[11][lane] = q2.w;
                    sm.td[12][lane] = q3.x; sm.td[13][lane] = q3.y; sm.td[14][lane] = q3.z; sm.td[15][lane] = q3.w;
                    sm.tri[lane] = (S32)((S64)tri - triBase);
                }
            }
            __syncwarp();
            U32 validMask = __ballot_sync(0xFFFFFFFFu, valid);

            // 2. Pixel coverage per triangle, two pixels per lane.
            const S32 qx = (lane & 7) << kSubpixelLog2;
            const S32 qy0 = (lane >> 3) << kSubpixelLog2;
            const S32 qy1 = qy0 + (4 << kSubpixelLog2);
            U32 myLo = 0, myHi = 0;
            for (U32 m = validMask; m; m &= m - 1) {
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
                U32 lo = __ballot_sync(0xFFFFFFFFu, c0);
                U32 hi = __ballot_sync(0xFFFFFFFFu, c1);
                if (kQuads) {
                    // quadCoverage (FineRaster.inl:401-406): bit of the quad's top-left pixel.
                    U64 c = ((U64)hi << 32) | lo;
                    c |= c >> 1;
                    c |= c >> 8;
                    c &= 0x0055005500550055ull;
                    lo = (U32)c; hi = (U32)(c >> 32);
                }
                if (lane == j) { myLo = lo; myHi = hi; }
            }
            // 3. Fragment compaction in submission order.
            S32 pop = (__popc(myLo) + __popc(myHi)) * (kQuads ? 4 : 1);
            S32 inc = pop;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                S32 t = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                if (lane >= o) inc += t;
            }
            sm.fragEnd[lane] = inc;
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
                if (act) {
                    // Triangle of fragment f: first j with fragEnd[j] > f.
                    int lo = 0, hi = 31;
                    while (lo < hi) {
                        int mid = (lo + hi) >> 1;
                        if (sm.fragEnd[mid] > f) hi = mid; else lo = mid + 1;
                    }
                    j = lo;
                    const S32 k = f - (sm.fragEnd[j] - (S32)((__popc(sm.covLo[j]) + __popc(sm.covHi[j])) * (kQuads ? 4 : 1)));
                    if (kQuads) {
                        int qbit = nthSetBit64(sm.covLo[j], sm.covHi[j], k >> 2);
                        pixel = qbit + (k & 1) + ((k & 2) << 2);  // findFragment, FineRaster.inl:417-427
                    } else {
                        pixel = nthSetBit64(sm.covLo[j], sm.covHi[j], k);
                    }
                    const S32 px = pixel & 7, py = pixel >> 3;
                    // Exact sample coverage.
#pragma unroll
                    for (int i = 0; i < NS; i++) {
                        const S32 sx = (px << kSubpixelLog2) + sampleOffsetX(S, i);
                        const S32 sy = (py << kSubpixelLog2) + sampleOffsetY(S, i);
                        bool c = true;
#pragma unroll
                        for (int e = 0; e < 3; e++) c = c && (sm.E[e][j] + sm.A[e][j] * sx + sm.B[e][j] * sy >= 0);
                        if (c) sampleMask |= 1u << i;
                    }
                    covered = sampleMask != 0;
                    if (!kQuads && !covered) act = false;
                    // Depth at the samples (FineRaster.inl:695, 1047, 1096).
                    const U32 X = (U32)(tx * 8 + px), Y = (U32)(ty * 8 + py);
                    if (kDepth) {
                        const U32 zx = sm.td[0][j], zy = sm.td[1][j], zb = sm.td[2][j];
                        bool anyPass = false;
                        if (S == 0) {
                            dz[0] = zx * X + zy * Y + zb;
                        } else {
                            const U32 zbase = ((zx * X + zy * Y) << S) + zb;
#pragma unroll
                            for (int i = 0; i < NS; i++) dz[i] = zx * (U32)msaaPatternX(S, i) + zy * (U32)i + zbase;
                        }
                        const int rowBase = py * 8 * NS + px;
#pragma unroll
                        for (int i = 0; i < NS; i++)
                            if ((sampleMask >> i & 1) && dz[i] < sm.depth[rowBase + i * 8]) anyPass = true;
                        if (!kQuads && !anyPass) act = false;
                        if (kQuads && !anyPass) covered = false;
                    }
                }
                // Shade.
                const U32 shadeMask = __ballot_sync(0xFFFFFFFFu, act);
                U32 src = 0;
                bool discard = true;
                if (act) {
                    const S32 px = pixel & 7, py = pixel >> 3;
                    const S32 X = tx * 8 + px, Y = ty * 8 + py;
                    FS fs;
                    fs.m_triIdx = sm.tri[j];
                    fs.m_vertIdx = FW::Vec3i((S32)sm.td[13][j], (S32)sm.td[14][j], (S32)sm.td[15][j]);
                    fs.m_pixelPos = FW::Vec2i(X, Y);
                    fs.m_vertexBytes = stride4 * 16;
                    fs.m_shared = sm.shared;
                    fs.m_vertices = verts;
                    fs.m_laneMask = shadeMask;
                    fs.m_color = 0xFF0000FFu;
                    fs.m_discard = false;
                    if (!kLerp) {
                        fs.m_center = FW::Vec3f(0.0f, 0.0f, 1.0f);
                        fs.m_centerDX = FW::Vec3f(0.0f);
                        fs.m_centerDY = FW::Vec3f(0.0f);
                        fs.m_centroid = fs.m_center;
                        fs.m_centroidDX = fs.m_centerDX;
                        fs.m_centroidDY = fs.m_centerDY;
                    } else {
                        U32 w[3] = {sm.td[4][j], sm.td[5][j], sm.td[6][j]};
                        U32 u[3] = {sm.td[7][j], sm.td[8][j], sm.td[9][j]};
                        U32 v[3] = {sm.td[10][j], sm.td[11][j], sm.td[12][j]};
                        computeBarys<S>(fs.m_center, fs.m_centerDX, fs.m_centerDY, w, u, v, (X * 2 + 1) << S, (Y * 2 + 1) << S);
                        if (S == 0) {
                            fs.m_centroid = fs.m_center;
                            fs.m_centroidDX = fs.m_centerDX;
                            fs.m_centroidDY = fs.m_centerDY;
                        } else {
                            U32 c = centroidCode(S, sampleMask);
                            computeBarys<S>(fs.m_centroid, fs.m_centroidDX, fs.m_centroidDY, w, u, v,
                                            (X << (S + 1)) + (S32)(c & 0xF), (Y << (S + 1)) + (S32)(c >> 4));
                        }
                    }
                    fs.run();
                    src = fs.m_color;
                    discard = fs.m_discard;
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
                            const S32 px = pixel & 7, py = pixel >> 3;
                            const int rowBase = py * 8 * NS + px;
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
                                bs.m_pixelPos = FW::Vec2i(tx * 8 + px, ty * 8 + py);
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

        // Write the tile back (FineRaster.inl:736-746).
        for (int w = lane; w < TW; w += 32) {
            S64 g = tileOrigin + (S64)(w / (8 * NS)) * rowWords + (w % (8 * NS));
            gColor[g] = sm.color[w];
            gDepth[g] = sm.depth[w];
        }
        __syncwarp();
    }
}

}  // namespace cr
