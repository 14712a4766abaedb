// binning.cu -- bin and coarse stages (stages 2 and 3 of 4).
//
// The reference bins with 16 persistent CTAs writing segmented linked lists
// per (bin, stream) and then merges the 16 streams per bin in triangle order
// (BinRaster.inl:19-469, CoarseRaster.inl:28-809). On GB300 both stages are
// count -> scan -> scatter passes over all SMs instead:
//
//   bin:    chunks of consecutive triangles, each taken by one warp (in
//           order, as warps free up). binCount counts (bin, chunk) entries,
//           binScan turns the counts into per-bin offsets in chunk order and
//           allocates each bin's contiguous list, binScatter writes the
//           entries. Every bin list comes out in submission order, with no
//           merge.
//   coarse: units of consecutive bin-list entries of one bin (sized on the
//           device once the bin lists are known), each taken by one warp,
//           with the same three passes over the tiles of the bin.
//
// Both stages walk their items 32 at a time (a group) and expand a group into
// (item, cell) pairs -- every cell of each item's bounding box -- dealt
// evenly over the lanes, so an item covering many cells costs its cell count
// / 32 iterations instead of holding up the whole warp. Pairs are taken 32 at
// a time in item order; the rank of a pair in its cell's list is the cell's
// running index plus the number of lower lanes on the same cell (a match on
// the cell index).
//
// List entries are triangle << 3 | subtriangle (7 = the triangle's own slot),
// as in the reference. Placement of a list in memory depends on atomics,
// its content and order do not.
#include "cudaraster/detail/binning.cuh"
#include "cudaraster/detail/launch.h"
#include "cudaraster/detail/per_device.h"

namespace cr {

constexpr int kBinThreads = 512;
constexpr int kBinWarps = kBinThreads / 32;

// Exclusive block scan over kBinThreads values; returns the exclusive prefix,
// total in *total. scratch >= kBinWarps + 1 ints.
__device__ __forceinline__ S32 blockExclusiveScan(S32 v, S32* scratch, S32* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    S32 inc = warpInclusiveScan(v);
    if (lane == 31) scratch[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        S32 w = (lane < kBinWarps) ? scratch[lane] : 0;
        S32 wi = warpInclusiveScan(w);
        if (lane < kBinWarps) scratch[lane] = wi - w;
        if (lane == kBinWarps - 1) scratch[kBinWarps] = wi;
    }
    __syncthreads();
    S32 r = scratch[warp] + inc - v;
    *total = scratch[kBinWarps];
    __syncthreads();
    return r;
}

// Geometry of a cell grid (bins of the viewport, or tiles inside one bin).
struct Grid {
    S32 halfW, halfH, cellLog2;
    bool centerOnly;          // one sample per pixel: boxes of pixel centres (cellBox)
    S32 cx0, cy0, cx1, cy1;   // clamp window (inclusive)
    S32 stride;               // cells per row of the local index space
};

// The current group of a warp, one word per list item (lane).
struct GroupSmem {
    S32 incl[32];   // inclusive prefix of the entries' box tile counts
    U32 v[3][32];   // vertices, packed as in the triangle header
    U32 box[32];    // lx | ly << 9 | (w - 1) << 18 (local cells, < 512 each), bit 31: box of at most 2x2 cells
    U32 mul[32];    // ceil(2^32 / w) (0 for w = 1): cell k of the box is in row umulhi(k, mul)
    U32 entry[32];
};

// Publishes a group of up to 32 list items (lane i: item entry, if valid)
// with their cell boxes; returns the group's number of (item, cell) pairs
// and the lane's inclusive prefix of them in incl -- or -1 when no item has
// more than one cell, with the lane's own cell (or -1) in cell1.
__device__ __forceinline__ S32 stageItems(const DrawDev& d, const Grid& gr, bool valid, U32 entry, GroupSmem& gs,
                                          S32& incl, int& cell1) {
    const int lane = threadIdx.x & 31;
    S32 n = 0;
    CellBox b{};
    uint4 h = make_uint4(0u, 0u, 0u, 0u);
    if (valid) {
        h = __ldg(&d.triHeader[entrySlot(entry, d.triHeader)]);
        b = cellBox(geomFromHeader(h), gr.halfW, gr.halfH, gr.cellLog2, gr.cx0, gr.cy0, gr.cx1, gr.cy1, gr.centerOnly);
        n = b.count();
    }
    gs.entry[lane] = entry;
    // Every item in at most one cell (the common case for small triangles):
    // the pairs are the items themselves, no expansion needed.
    if (__all_sync(0xFFFFFFFFu, n <= 1)) {
        cell1 = n == 1 ? (b.ly - gr.cy0) * gr.stride + (b.lx - gr.cx0) : -1;
        __syncwarp();
        return -1;
    }
    U32 box = 0, mul = 0;
    if (n > 0) {
        const U32 w = (U32)(b.hx - b.lx + 1);
        box = (U32)(b.lx - gr.cx0) | (U32)(b.ly - gr.cy0) << 9 | (w - 1u) << 18 | (b.small() ? 1u << 31 : 0u);
        mul = w > 1u ? 0xFFFFFFFFu / w + 1u : 0u;
    }
    incl = warpInclusiveScan(n);
    gs.incl[lane] = incl;
    gs.v[0][lane] = h.x;
    gs.v[1][lane] = h.y;
    gs.v[2][lane] = h.z;
    gs.box[lane] = box;
    gs.mul[lane] = mul;
    __syncwarp();
    return __shfl_sync(0xFFFFFFFFu, incl, 31);
}

// Pair p of the group (p below the group's pair count): its item j and its
// cell in the grid's local index space; returns whether the item's triangle
// may touch the cell (always, for boxes of at most 2x2 cells). The quotient
// k / w = umulhi(k, ceil(2^32 / w)) is exact for k * w < 2^32 (boxes have at
// most 512 x 512 cells).
__device__ __forceinline__ bool pairCell(const GroupSmem& gs, const Grid& gr, S32 p, int& j, int& cell) {
    int jj = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1)
        if (gs.incl[jj + s - 1] <= p) jj += s;
    const S32 k = p - (jj ? gs.incl[jj - 1] : 0);
    const U32 box = gs.box[jj];
    const S32 w = (S32)((box >> 18) & 0x1FFu) + 1;
    const U32 mul = gs.mul[jj];
    const S32 q = mul ? (S32)__umulhi((U32)k, mul) : k;
    const S32 lx = (S32)(box & 0x1FFu) + k - q * w;
    const S32 ly = (S32)((box >> 9) & 0x1FFu) + q;
    j = jj;
    cell = ly * gr.stride + lx;
    if (box >> 31) return true;
    const TriGeom g = geomFromHeader(make_uint4(gs.v[0][jj], gs.v[1][jj], gs.v[2][jj], 0u));
    const S32 side = 1 << gr.cellLog2;
    const S32 rx0 = ((gr.cx0 + lx) << gr.cellLog2) - gr.halfW, ry0 = ((gr.cy0 + ly) << gr.cellLog2) - gr.halfH;
    return triTouchesRect(g, rx0, ry0, rx0 + side - 1, ry0 + side - 1);
}

// Next work item (bin chunk or coarse unit) for this warp, taken in order
// from a counter; uniform across the warp.
__device__ __forceinline__ int warpNextUnit(S32* counter) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(counter, 1);
    return __shfl_sync(0xFFFFFFFFu, u, 0);
}

__device__ __forceinline__ Grid binGrid(const InstanceDev* in, int binLog2) {
    Grid gr;
    gr.halfW = __ldg(&in->width) << (kSubpixelLog2 - 1);
    gr.halfH = __ldg(&in->height) << (kSubpixelLog2 - 1);
    gr.cellLog2 = binLog2 + kTileLog2 + kSubpixelLog2;
    gr.centerOnly = __ldg(&in->samplesLog2) == 0;
    gr.cx0 = 0;
    gr.cy0 = 0;
    gr.cx1 = __ldg(&in->widthBins) - 1;
    gr.cy1 = __ldg(&in->heightBins) - 1;
    gr.stride = __ldg(&in->widthBins);
    return gr;
}

// ------------------------------------------------------------------ bin

// A warp's slice of a chunk streams its subtriangle items through a ring in
// shared memory; culled triangles carry none. Items keep (triangle,
// subtriangle) order.
constexpr int kRing = 256;

// Appends the items of the slice's next triangles until the ring holds at
// least 32 items or the slice is exhausted: four triangles per lane, or one
// per lane when four would overflow the ring (32 triangles carry at most 224
// items, which always fit behind fewer than 32). next and fill are uniform.
__device__ __forceinline__ void refillRing(const DrawDev& d, S64& next, S64 end, U32* ring, S32 head, S32& fill) {
    const int lane = threadIdx.x & 31;
    while (fill < 32 && next < end) {
        const S64 t = next + (S64)lane * 4;
        int n[4];
        int sum = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            n[j] = (t + j < end) ? d.triSubtris[t + j] : 0;
            sum += n[j];
        }
        const S32 incl = warpInclusiveScan(sum);
        const S32 total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        if (fill + total <= kRing) {
            S32 pos = head + fill + incl - sum;
#pragma unroll
            for (int j = 0; j < 4; j++)
                for (int s = 0; s < n[j]; s++) ring[(pos++) & (kRing - 1)] = ((U32)(t + j) << 3) | (U32)(n[j] == 1 ? 7 : s);
            fill += total;
            next += 32 * 4;
        } else {
            const S64 t1 = next + lane;
            const int m = (t1 < end) ? d.triSubtris[t1] : 0;
            const S32 incl1 = warpInclusiveScan(m);
            S32 pos = head + fill + incl1 - m;
            for (int s = 0; s < m; s++) ring[(pos++) & (kRing - 1)] = ((U32)t1 << 3) | (U32)(m == 1 ? 7 : s);
            fill += __shfl_sync(0xFFFFFFFFu, incl1, 31);
            next += 32;
        }
    }
    __syncwarp();
}

// Walks the items of triangles [next, end) over the bin grid: fn(hit, cell,
// j, peers) is called by every lane for each batch of 32 pairs, hit telling
// whether the lane's pair touches its cell, j the pair's lane in the group
// (its item) and peers the lanes of the batch on the same cell.
template <class Fn>
__device__ __forceinline__ void walkSlice(const DrawDev& d, const Grid& gr, S64 next, S64 end, U32* ring,
                                          GroupSmem& gs, Fn fn) {
    const int lane = threadIdx.x & 31;
    S32 head = 0, fill = 0;
    for (;;) {
        refillRing(d, next, end, ring, head, fill);
        if (fill == 0) break;
        const int g = min(fill, 32);
        const bool valid = lane < g;
        const U32 entry = valid ? ring[(head + lane) & (kRing - 1)] : 0u;
        head = (head + g) & (kRing - 1);
        fill -= g;
        S32 incl;
        int cell1;
        const S32 P = stageItems(d, gr, valid, entry, gs, incl, cell1);
        if (P < 0) {
            const bool hit = cell1 >= 0;
            fn(hit, cell1, lane, __match_any_sync(0xFFFFFFFFu, hit ? (U32)cell1 : 0x80000000u + (U32)lane));
        }
        for (S32 base = 0; base < P; base += 32) {
            const S32 p = base + lane;
            int j = 0, cell = 0;
            const bool hit = p < P && pairCell(gs, gr, p, j, cell);
            const U32 peers = __match_any_sync(0xFFFFFFFFu, hit ? (U32)cell : 0x80000000u + (U32)lane);
            fn(hit, cell, j, peers);
        }
        __syncwarp();
    }
}

// Bin count / scatter CTAs: warps work independently, one chunk at a time.
constexpr int kWalkThreads = 256;
constexpr int kWalkWarps = kWalkThreads / 32;

struct ChunkInfo {
    const InstanceDev* in;
    int local;      // chunk index inside its instance
    int nb;         // bins of the instance
    S64 t0, t1;     // triangles of the chunk
};

__device__ __forceinline__ ChunkInfo chunkInfo(const DrawDev& d, int chunk) {
    ChunkInfo c;
    c.in = &d.inst[findInstance(d.chunkPrefix, d.numInstances, chunk)];
    c.local = chunk - __ldg(&c.in->chunkBase);
    c.nb = __ldg(&c.in->widthBins) * __ldg(&c.in->heightBins);
    const S64 triBase = __ldg(&c.in->triBase);
    c.t0 = triBase + (S64)c.local * __ldg(&c.in->chunkTris);
    c.t1 = min(c.t0 + __ldg(&c.in->chunkTris), triBase + __ldg(&c.in->numTris));
    return c;
}

// Persistent warps over chunks: each chunk's entry count per bin, written to
// the (bin, chunk) matrix where not zero (the matrix is zero between draws),
// and, when d.binStageCap > 0, its (bin, entry) pairs in list order for the
// scatter pass (as many as fit; their total in binStageCount).
__global__ void __launch_bounds__(kWalkThreads) binCountKernel(DrawDev d) {
    pdlWait();
    pdlTrigger();
    extern __shared__ S32 s_cells[];   // [kWalkWarps][maxBins]
    __shared__ U32 s_ring[kWalkWarps][kRing];
    __shared__ GroupSmem s_group[kWalkWarps];
    if (__ldg(&d.counters->overflow) & kOverflowSubtris) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const U32 ltMask = (1u << lane) - 1u;
    S32* cnt = s_cells + warp * d.maxBins;
    GroupSmem& gs = s_group[warp];
    for (;;) {
        const int chunk = warpNextUnit(&d.counters->binWork[0]);
        if (chunk >= d.totalChunks) break;
        const ChunkInfo c = chunkInfo(d, chunk);
        const Grid gr = binGrid(c.in, d.binLog2);
        for (int b = lane; b < c.nb; b += 32) cnt[b] = 0;
        __syncwarp();
        U64* stage = d.binStage + (S64)chunk * d.binStageCap;
        S32 staged = 0;   // pairs of the chunk so far (uniform)
        walkSlice(d, gr, c.t0, c.t1, s_ring[warp], gs, [&](bool hit, int cell, int j, U32 peers) {
            if (hit && (peers >> lane) == 1u) cnt[cell] += __popc(peers);
            if (d.binStageCap > 0) {
                const U32 hits = __ballot_sync(0xFFFFFFFFu, hit);
                const S32 pos = staged + __popc(hits & ltMask);
                if (hit && pos < d.binStageCap) stage[pos] = (U64)(U32)cell << 32 | gs.entry[j];
                staged += __popc(hits);
            }
        });
        if (lane == 0 && d.binStageCap > 0) d.binStageCount[chunk] = staged;
        S32* out = d.chunkBinCount + __ldg(&c.in->chunkCountBase) + c.local;
        const S64 nc = __ldg(&c.in->numChunks);
        for (int b = lane; b < c.nb; b += 32) {
            const S32 v = cnt[b];
            if (v) out[b * nc] = v;
        }
        __syncwarp();
    }
}

// Run by the last bin-scan CTA to finish, once every bin's entry count is
// known: the coarse unit size (the caller's, or the smallest power of two
// from 64 that gives at most unitTarget units and fits maxUnits) and each
// bin's first unit. Contains barriers; the whole CTA calls it.
__device__ __forceinline__ void planUnits(const DrawDev& d, S32* s_scratch) {
    const S64 total = __ldcg(&d.counters->binEntries);
    S64 U = d.unitEntries;
    if (U <= 0) {
        const S64 room = max((S64)1, d.maxUnits - d.totalBins - 1);
        U = 64;
        while (U < 4096 && total > (S64)max(d.unitTarget, 1) * U) U *= 2;
        while (total > room * U && U < ((S64)1 << 30)) U *= 2;
    }
    S32 carry = 0;
    for (int b0 = 0; b0 < d.totalBins; b0 += kBinThreads) {
        const int b = b0 + threadIdx.x;
        const U32 c = b < d.totalBins ? (U32)__ldcg(&d.binCount[b]) : 0u;
        const S32 n = (S32)(c / (U32)U + (c % (U32)U != 0u));
        S32 tot;
        const S32 ex = blockExclusiveScan(n, s_scratch, &tot);
        if (b < d.totalBins) d.binUnitFirst[b] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) {
        d.counters->unitEntries = (S32)U;
        d.counters->numUnits = carry;
    }
}

// One CTA per global bin: chunk-order exclusive offsets and list allocation;
// the last CTA to finish plans the coarse units.
__global__ void __launch_bounds__(kBinThreads) binScanKernel(DrawDev d) {
    pdlWait();
    pdlTrigger();
    __shared__ S32 s_scratch[kBinWarps + 1];
    __shared__ int s_inst;
    __shared__ bool s_last;
    if (__ldg(&d.counters->overflow) & kOverflowSubtris) return;
    const int gb = blockIdx.x;
    if (threadIdx.x == 0) s_inst = findInstance(d.binPrefix, d.numInstances, gb);
    __syncthreads();
    const InstanceDev* in = &d.inst[s_inst];
    const int nb = __ldg(&in->widthBins) * __ldg(&in->heightBins);
    const int b = gb - __ldg(&in->binBase);
    const int nc = __ldg(&in->numChunks);
    S32* counts = d.chunkBinCount + __ldg(&in->chunkCountBase) + (S64)b * nc;
    S32* offs = d.chunkBinOffset + __ldg(&in->chunkCountBase) + b;
    // Eight consecutive chunks per thread, loaded before they are summed.
    constexpr int kPer = 8;
    S32 carry = 0;
    for (int c0 = 0; c0 < nc; c0 += kBinThreads * kPer) {
        const int cb = c0 + threadIdx.x * kPer;
        S32 v[kPer];
#pragma unroll
        for (int k = 0; k < kPer; k++) v[k] = (cb + k < nc) ? counts[cb + k] : 0;
        S32 sum = 0;
#pragma unroll
        for (int k = 0; k < kPer; k++) sum += v[k];
        S32 tot;
        S32 ex = carry + blockExclusiveScan(sum, s_scratch, &tot);
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            if (v[k]) {
                counts[cb + k] = 0;
                offs[(S64)(cb + k) * nb] = ex;
                ex += v[k];
            }
        }
        carry += tot;
    }
    if (threadIdx.x == 0) {
        S32 start = atomicAdd(&d.counters->binEntries, carry);
        if ((S64)start + carry > d.maxBinEntries) atomicOr(&d.counters->overflow, kOverflowBin);
        d.binStart[gb] = start;
        d.binCount[gb] = carry;
        __threadfence();
        s_last = atomicAdd(&d.counters->binsDone, 1) == d.totalBins - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        planUnits(d, s_scratch);
    }
}

// Persistent warps over chunks: writes each chunk's entries into the bin
// lists, from the chunk's offset in every bin it touches: from the pairs the
// count pass recorded, 32 at a time (a pair's rank in its bin is the bin's
// running index plus the lower lanes of the batch on the same bin), or, for a
// chunk whose pairs did not fit, by walking its triangles again.
__global__ void __launch_bounds__(kWalkThreads) binScatterKernel(DrawDev d) {
    pdlWait();
    pdlTrigger();
    extern __shared__ S32 s_cells[];   // [kWalkWarps][maxBins]: next list index per bin
    __shared__ U32 s_ring[kWalkWarps][kRing];
    __shared__ GroupSmem s_group[kWalkWarps];
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin)) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const U32 ltMask = (1u << lane) - 1u;
    S32* run = s_cells + warp * d.maxBins;
    GroupSmem& gs = s_group[warp];
    for (;;) {
        const int chunk = warpNextUnit(&d.counters->binWork[1]);
        if (chunk >= d.totalChunks) break;
        const ChunkInfo c = chunkInfo(d, chunk);
        const Grid gr = binGrid(c.in, d.binLog2);
        // Offsets of bins the chunk does not touch are stale and never used.
        const S32* offs = d.chunkBinOffset + __ldg(&c.in->chunkCountBase) + (S64)c.local * c.nb;
        const S32 binBase = __ldg(&c.in->binBase);
        for (int b = lane; b < c.nb; b += 32) run[b] = __ldg(&d.binStart[binBase + b]) + __ldg(&offs[b]);
        __syncwarp();
        const S32 staged = d.binStageCap > 0 ? __ldcg(&d.binStageCount[chunk]) : -1;
        if (staged >= 0 && staged <= d.binStageCap) {
            const U64* stage = d.binStage + (S64)chunk * d.binStageCap;
            U64 next = lane < staged ? __ldcg(&stage[lane]) : 0ull;   // the next batch loads during this one
            for (S32 i0 = 0; i0 < staged; i0 += 32) {
                const bool valid = i0 + lane < staged;
                const U64 pr = next;
                if (i0 + 32 + lane < staged) next = __ldcg(&stage[i0 + 32 + lane]);
                const int cell = (int)(pr >> 32);
                const U32 peers = __match_any_sync(0xFFFFFFFFu, valid ? (U32)cell : 0x80000000u + (U32)lane);
                if (valid) {
                    const S64 idx = (S64)run[cell] + __popc(peers & ltMask);
                    if (idx < d.maxBinEntries) d.binList[idx] = (U32)pr;
                }
                __syncwarp();
                if (valid && (peers >> lane) == 1u) run[cell] += __popc(peers);
                __syncwarp();
            }
            continue;
        }
        walkSlice(d, gr, c.t0, c.t1, s_ring[warp], gs, [&](bool hit, int cell, int j, U32 peers) {
            if (hit) {
                const S64 idx = (S64)run[cell] + __popc(peers & ltMask);
                if (idx < d.maxBinEntries) d.binList[idx] = gs.entry[j];
            }
            __syncwarp();
            if (hit && (peers >> lane) == 1u) run[cell] += __popc(peers);
            __syncwarp();
        });
    }
}

// --------------------------------------------------------------- coarse
//
// A coarse unit (up to unitEntries consecutive entries of one bin list) is
// taken by one warp, which walks it 32 entries (a group) at a time. No
// CTA-wide barrier is involved: units, groups and ranks are all warp-local.

constexpr int kCoarseThreads = 256;
constexpr int kCoarseWarps = kCoarseThreads / 32;

struct UnitInfo {
    const InstanceDev* in;
    S32 gb, seg, bx, by, e0, e1;
};

// Unit u: the last bin whose first unit is at most u (bins without units
// share their first unit with the next bin), and its entry range.
__device__ __forceinline__ void loadUnit(const DrawDev& d, int u, S32 unitEntries, UnitInfo& ui) {
    int lo = 0, hi = d.totalBins - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&d.binUnitFirst[mid]) <= u) lo = mid; else hi = mid - 1;
    }
    ui.gb = lo;
    ui.in = &d.inst[findInstance(d.binPrefix, d.numInstances, ui.gb)];
    ui.seg = u - __ldg(&d.binUnitFirst[lo]);
    const S32 b = ui.gb - __ldg(&ui.in->binBase);
    const S32 wb = __ldg(&ui.in->widthBins);
    ui.bx = b % wb;
    ui.by = b / wb;
    const S32 start = __ldg(&d.binStart[ui.gb]), cnt = __ldg(&d.binCount[ui.gb]);
    ui.e0 = start + ui.seg * unitEntries;
    ui.e1 = min(ui.e0 + unitEntries, start + cnt);
}

__device__ __forceinline__ Grid tileGrid(const UnitInfo& ui, int binLog2) {
    Grid gr;
    const S32 side = 1 << binLog2;
    gr.halfW = __ldg(&ui.in->width) << (kSubpixelLog2 - 1);
    gr.halfH = __ldg(&ui.in->height) << (kSubpixelLog2 - 1);
    gr.cellLog2 = kTileLog2 + kSubpixelLog2;
    gr.centerOnly = __ldg(&ui.in->samplesLog2) == 0;
    gr.cx0 = ui.bx << binLog2;
    gr.cy0 = ui.by << binLog2;
    gr.cx1 = min(gr.cx0 + side - 1, __ldg(&ui.in->widthTiles) - 1);
    gr.cy1 = min(gr.cy0 + side - 1, __ldg(&ui.in->heightTiles) - 1);
    gr.stride = side;
    return gr;
}

// Persistent warps over coarse units (taken dynamically): per-unit tile
// counts, and, for units below d.tileStageUnits, their (tile, entry) pairs in
// list order for the scatter pass (as many as fit; their total in
// tileStageCount).
__global__ void __launch_bounds__(kCoarseThreads) coarseCountKernel(DrawDev d) {
    pdlWait();
    pdlTrigger();
    extern __shared__ S32 smem[];
    __shared__ GroupSmem s_group[kCoarseWarps];
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tpb = 1 << (2 * d.binLog2);
    S32* cnt = smem + warp * tpb;
    GroupSmem& gs = s_group[warp];
    const U32 ltMask = (1u << lane) - 1u;
    const S32 numUnits = (S32)min((S64)__ldg(&d.counters->numUnits), d.maxUnits);
    const S32 unitEntries = __ldg(&d.counters->unitEntries);
    for (;;) {
        const int u = warpNextUnit(&d.counters->coarseWork[0]);   // count pass
        if (u >= numUnits) break;
        UnitInfo ui;
        loadUnit(d, u, unitEntries, ui);
        const Grid gr = tileGrid(ui, d.binLog2);
        for (int t = lane; t < tpb; t += 32) cnt[t] = 0;
        __syncwarp();
        const bool record = u < d.tileStageUnits;
        U64* stage = d.tileStage + (S64)u * d.tileStageCap;
        S32 staged = 0;   // pairs of the unit so far (uniform)
        // Records the batch's hits in lane order, which is list order.
        auto recordHits = [&](bool hit, int cell, U32 entry) {
            const U32 hits = __ballot_sync(0xFFFFFFFFu, hit);
            const S32 pos = staged + __popc(hits & ltMask);
            if (hit && pos < d.tileStageCap) stage[pos] = (U64)(U32)cell << 32 | entry;
            staged += __popc(hits);
        };
        for (S32 e0 = ui.e0; e0 < ui.e1; e0 += 32) {
            S32 incl;
            int cell1;
            const bool valid = e0 + lane < ui.e1;
            const S32 P = stageItems(d, gr, valid, valid ? __ldg(&d.binList[e0 + lane]) : 0u, gs, incl, cell1);
            if (P < 0) {
                if (cell1 >= 0) atomicAdd(&cnt[cell1], 1);
                if (record) recordHits(cell1 >= 0, cell1, gs.entry[lane]);
            }
            for (S32 base = 0; base < P; base += 32) {
                const S32 p = base + lane;
                int j = 0, cell = 0;
                const bool hit = p < P && pairCell(gs, gr, p, j, cell);
                if (hit) atomicAdd(&cnt[cell], 1);
                if (record) recordHits(hit, cell, gs.entry[j]);
            }
            __syncwarp();
        }
        if (lane == 0 && record) d.tileStageCount[u] = staged;
        S32* out = d.unitTileCount + (S64)u * tpb;
        for (int t = lane; t < tpb; t += 32) out[t] = cnt[t];
        __syncwarp();
    }
}

// One CTA per global bin: unit-order offsets per tile and tile list
// allocation. Each warp takes a contiguous slice of the bin's units: it sums
// its slice per tile, the slice sums are scanned across warps per tile, and
// each warp then writes its slice's running offsets.
__global__ void __launch_bounds__(kBinThreads) coarseScanKernel(DrawDev d) {
    pdlWait();
    pdlTrigger();
    extern __shared__ S32 s_part[];   // [kBinWarps][tpb]: slice sums, then slice starts
    __shared__ S32 s_scratch[kBinWarps + 1];
    __shared__ int s_inst;
    __shared__ S32 s_base;
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin)) return;
    const int gb = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) s_inst = findInstance(d.binPrefix, d.numInstances, gb);
    __syncthreads();
    const InstanceDev* in = &d.inst[s_inst];
    const int tpb = 1 << (2 * d.binLog2);
    const S32 side = 1 << d.binLog2;
    const S32 b = gb - __ldg(&in->binBase);
    const S32 wb = __ldg(&in->widthBins);
    const S32 bx = b % wb, by = b / wb;
    const S32 wt = __ldg(&in->widthTiles), ht = __ldg(&in->heightTiles);
    const S32 tileBase = __ldg(&in->tileBase);
    const S32 cnt = __ldg(&d.binCount[gb]);
    const S32 unitEntries = __ldg(&d.counters->unitEntries);
    const S32 units = (cnt + unitEntries - 1) / unitEntries;
    S32* counts = d.unitTileCount + (S64)__ldg(&d.binUnitFirst[gb]) * tpb;
    const S32 per = (units + kBinWarps - 1) / kBinWarps;
    const S32 k0 = min(warp * per, units), k1 = min(k0 + per, units);
    for (int t = lane; t < tpb; t += 32) {
        S32 acc = 0;
        for (S32 k = k0; k < k1; k++) acc += counts[(S64)k * tpb + t];
        s_part[warp * tpb + t] = acc;
    }
    __syncthreads();
    S32 carry = 0;
    for (int t0 = 0; t0 < tpb; t0 += kBinThreads) {
        const int t = t0 + threadIdx.x;
        S32 acc = 0;
        if (t < tpb) {
            for (int w = 0; w < kBinWarps; w++) {
                const S32 v = s_part[w * tpb + t];
                s_part[w * tpb + t] = acc;
                acc += v;
            }
        }
        S32 tot;
        const S32 ex = blockExclusiveScan(acc, s_scratch, &tot);
        if (t < tpb) {
            const S32 tx = (bx << d.binLog2) + (t & (side - 1));
            const S32 ty = (by << d.binLog2) + (t >> d.binLog2);
            if (tx < wt && ty < ht) {
                const S32 g = tileBase + ty * wt + tx;
                d.tileCount[g] = acc;
                d.tileStart[g] = carry + ex;   // relative; rebased below
            }
        }
        carry += tot;
    }
    if (threadIdx.x == 0) {
        const S32 base = atomicAdd(&d.counters->tileEntries, carry);
        if ((S64)base + carry > d.maxTileEntries) atomicOr(&d.counters->overflow, kOverflowTile);
        s_base = base;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < tpb; t += kBinThreads) {
        const S32 tx = (bx << d.binLog2) + (t & (side - 1));
        const S32 ty = (by << d.binLog2) + (t >> d.binLog2);
        if (tx < wt && ty < ht) d.tileStart[tileBase + ty * wt + tx] += s_base;
    }
    for (int t = lane; t < tpb; t += 32) {
        S32 run = s_part[warp * tpb + t];
        for (S32 k = k0; k < k1; k++) {
            S32* p = &counts[(S64)k * tpb + t];
            const S32 c = *p;
            *p = run;
            run += c;
        }
    }
}

// Persistent warps over coarse units (taken dynamically): writes tile list
// entries, from the pairs the count pass recorded or, for a unit whose pairs
// were not recorded, by walking its entries again. Pairs are taken 32 at a
// time in list order; the rank of a pair in its tile list is the tile's
// running index plus the number of lower lanes of the batch on the same tile
// (a match on the tile index).
__global__ void __launch_bounds__(kCoarseThreads) coarseScatterKernel(DrawDev d) {
    pdlWait();
    pdlTrigger();
    extern __shared__ S32 smem[];
    __shared__ GroupSmem s_group[kCoarseWarps];
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin | kOverflowTile)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const U32 ltMask = (1u << lane) - 1u;
    const int tpb = 1 << (2 * d.binLog2);
    const S32 side = 1 << d.binLog2;
    S32* run = smem + (size_t)warp * tpb;
    GroupSmem& gs = s_group[warp];
    const S32 numUnits = (S32)min((S64)__ldg(&d.counters->numUnits), d.maxUnits);
    const S32 unitEntries = __ldg(&d.counters->unitEntries);
    for (;;) {
        const int u = warpNextUnit(&d.counters->coarseWork[1]);
        if (u >= numUnits) break;
        UnitInfo ui;
        loadUnit(d, u, unitEntries, ui);
        const Grid gr = tileGrid(ui, d.binLog2);
        const S32 wt = __ldg(&ui.in->widthTiles);
        const S32 tileBase = __ldg(&ui.in->tileBase);
        const S32* unitCount = d.unitTileCount + (S64)u * tpb;
        for (int t = lane; t < tpb; t += 32) {
            const S32 tx = gr.cx0 + (t & (side - 1)), ty = gr.cy0 + (t >> d.binLog2);
            S32 v = 0;
            if (tx <= gr.cx1 && ty <= gr.cy1) v = __ldg(&d.tileStart[tileBase + ty * wt + tx]) + __ldg(&unitCount[t]);
            run[t] = v;
        }
        __syncwarp();
        const S32 staged = u < d.tileStageUnits ? __ldcg(&d.tileStageCount[u]) : -1;
        if (staged >= 0 && staged <= d.tileStageCap) {
            const U64* stage = d.tileStage + (S64)u * d.tileStageCap;
            U64 next = lane < staged ? __ldcg(&stage[lane]) : 0ull;   // the next batch loads during this one
            for (S32 i0 = 0; i0 < staged; i0 += 32) {
                const bool valid = i0 + lane < staged;
                const U64 pr = next;
                if (i0 + 32 + lane < staged) next = __ldcg(&stage[i0 + 32 + lane]);
                const int cell = (int)(pr >> 32);
                const U32 peers = __match_any_sync(0xFFFFFFFFu, valid ? (U32)cell : 0x80000000u + (U32)lane);
                if (valid) {
                    const S64 idx = (S64)run[cell] + __popc(peers & ltMask);
                    if (idx < d.maxTileEntries) d.tileList[idx] = (U32)pr;
                }
                __syncwarp();
                if (valid && (peers >> lane) == 1u) run[cell] += __popc(peers);
                __syncwarp();
            }
            continue;
        }
        for (S32 e0 = ui.e0; e0 < ui.e1; e0 += 32) {
            S32 incl;
            int cell1;
            const bool valid = e0 + lane < ui.e1;
            const S32 P = stageItems(d, gr, valid, valid ? __ldg(&d.binList[e0 + lane]) : 0u, gs, incl, cell1);
            if (P < 0) {
                const bool hit = cell1 >= 0;
                const U32 peers = __match_any_sync(0xFFFFFFFFu, hit ? (U32)cell1 : 0x80000000u + (U32)lane);
                if (hit) {
                    const S64 idx = (S64)run[cell1] + __popc(peers & ltMask);
                    if (idx < d.maxTileEntries) d.tileList[idx] = gs.entry[lane];
                }
                __syncwarp();
                if (hit && (peers >> lane) == 1u) run[cell1] += __popc(peers);
                __syncwarp();
            }
            for (S32 base = 0; base < P; base += 32) {
                const S32 p = base + lane;
                int j = 0, cell = 0;
                const bool hit = p < P && pairCell(gs, gr, p, j, cell);
                const U32 peers = __match_any_sync(0xFFFFFFFFu, hit ? (U32)cell : 0x80000000u + (U32)lane);
                if (hit) {
                    const S64 idx = (S64)run[cell] + __popc(peers & ltMask);
                    if (idx < d.maxTileEntries) d.tileList[idx] = gs.entry[j];
                }
                __syncwarp();
                if (hit && (peers >> lane) == 1u) run[cell] += __popc(peers);
                __syncwarp();
            }
        }
    }
}

// ------------------------------------------------------------ launchers

size_t binWalkSmem(int maxBins) { return sizeof(S32) * kWalkWarps * (size_t)maxBins; }
size_t coarseCountSmem(int binLog2) { return sizeof(S32) * kCoarseWarps * ((size_t)1 << (2 * binLog2)); }
size_t coarseScatterSmem(int binLog2) { return sizeof(S32) * kCoarseWarps * ((size_t)1 << (2 * binLog2)); }

cudaError_t launchBinning(const DrawDev& d, int maxBins, int numSMs, cudaStream_t stream, cudaEvent_t evCoarse) {
    // Shared-memory limits are per device: set them once on each device used.
    static OncePerDevice attributes;
    attributes.run([] {
        cudaFuncSetAttribute(binScatterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        cudaFuncSetAttribute(binCountKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        cudaFuncSetAttribute(coarseScatterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        cudaFuncSetAttribute(coarseCountKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        cudaFuncSetAttribute(coarseScanKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    });
    // Resident coarse CTAs per SM for bins of 8, 16 and 32 tiles a side.
    static IntsPerDevice<6> coarseCountCtas, coarseScatterCtas;
    const int bl = d.binLog2 >= 3 && d.binLog2 <= 5 ? d.binLog2 : 4;
    const int countCtas = coarseCountCtas.get(bl, [](int b) {
        int n = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, coarseCountKernel, kCoarseThreads, coarseCountSmem(b));
        return n > 0 ? n : 1;
    });
    const int scatterCtas = coarseScatterCtas.get(bl, [](int b) {
        int n = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, coarseScatterKernel, kCoarseThreads, coarseScatterSmem(b));
        return n > 0 ? n : 1;
    });
    // Units sized on the device: about two per resident coarse-scatter warp.
    DrawDev dl = d;
    dl.unitTarget = 2 * numSMs * scatterCtas * kCoarseWarps;
    // binScan also runs for a draw without triangles: it zeroes the bin counts.
    // Persistent bin warps: as many CTAs as are resident at once, and no more
    // than the draw's chunks can keep busy.
    dl.maxBins = maxBins;
    const int walkSmem = (int)binWalkSmem(maxBins);
    static IntsPerDevice<1025> walkCtasFor;   // resident bin CTAs per SM, by bins of the largest instance
    const int mb = maxBins >= 1 && maxBins <= 1024 ? maxBins : 1024;
    const int walkCtas = walkCtasFor.get(mb, [](int bins) {
        int n = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, binScatterKernel, kWalkThreads, (int)binWalkSmem(bins));
        return n > 0 ? n : 1;
    });
    const int walkGrid = (int)min((S64)numSMs * walkCtas, (S64)(dl.totalChunks + kWalkWarps - 1) / kWalkWarps);
    cudaError_t e = cudaSuccess;
    if (dl.totalChunks > 0) e = launchKernel(binCountKernel, walkGrid, kWalkThreads, walkSmem, stream, true, dl);
    if (e == cudaSuccess) e = launchKernel(binScanKernel, dl.totalBins, kBinThreads, 0, stream, true, dl);
    if (e == cudaSuccess && dl.totalChunks > 0)
        e = launchKernel(binScatterKernel, walkGrid, kWalkThreads, walkSmem, stream, true, dl);
    if (e == cudaSuccess && evCoarse) e = cudaEventRecord(evCoarse, stream);
    if (e != cudaSuccess) return e;
    // Persistent coarse warps: as many CTAs as are resident at once, and no
    // more than the draw's units can keep busy.
    const S64 unitCtas = (dl.maxUnits + kCoarseWarps - 1) / kCoarseWarps;
    const int countGrid = (int)min((S64)numSMs * countCtas, unitCtas);
    const int scatterGrid = (int)min((S64)numSMs * scatterCtas, unitCtas);
    e = launchKernel(coarseCountKernel, countGrid, kCoarseThreads, coarseCountSmem(dl.binLog2), stream, true, dl);
    if (e == cudaSuccess)
        e = launchKernel(coarseScanKernel, dl.totalBins, kBinThreads,
                         sizeof(S32) * kBinWarps * ((size_t)1 << (2 * dl.binLog2)), stream, true, dl);
    if (e == cudaSuccess)
        e = launchKernel(coarseScatterKernel, scatterGrid, kCoarseThreads, coarseScatterSmem(dl.binLog2), stream, true,
                         dl);
    return e;
}

}  // namespace cr
