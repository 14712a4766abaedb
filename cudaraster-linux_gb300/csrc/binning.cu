// binning.cu -- bin and coarse stages (stages 2 and 3 of 4).
//
// The reference bins with 16 persistent CTAs writing segmented linked lists
// per (bin, stream) and then merges the 16 streams per bin in triangle order
// (BinRaster.inl:19-469, CoarseRaster.inl:28-809). On GB300 both stages are
// count -> scan -> scatter passes over all SMs instead:
//
//   bin:    chunks of consecutive triangles. binCount counts (chunk, bin)
//           entries, binScan turns the counts into per-bin offsets in chunk
//           order and allocates each bin's contiguous list, binScatter writes
//           the entries ranked inside each 512-item round by per-warp ballot
//           masks. Every bin list comes out in submission order, with no merge.
//   coarse: units of consecutive bin-list entries of one bin (sized on the
//           device once the bin lists are known), each taken by one warp,
//           with the same three passes over the tiles of the bin.
//
// In every bin round, an item whose bounding box spans more than kSmallCells
// bins is dealt to a warp (one bin per lane) instead of being walked by its
// own thread, so a few huge triangles do not serialise a round.
//
// List entries are triangle << 3 | subtriangle (7 = the triangle's own slot),
// as in the reference. Placement of a list in memory depends on atomics,
// its content and order do not.
#include "cudaraster/detail/binning.cuh"

namespace cr {

constexpr int kBinThreads = 512;
constexpr int kBinWarps = kBinThreads / 32;
constexpr int kMaxSubtrisPerTri = 7;
constexpr int kSmallCells = 8;

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
    S32 cx0, cy0, cx1, cy1;   // clamp window (inclusive)
    S32 stride;               // cells per row of the local index space
};

__device__ __forceinline__ int cellIndex(const Grid& gr, S32 cx, S32 cy) {
    return (cy - gr.cy0) * gr.stride + (cx - gr.cx0);
}

// Items too large for their own thread, walked by a whole warp. Vertices and
// box corners are kept as 16-bit pairs (snapped coordinates are S16, cell
// coordinates below 2^15).
struct BigItem {
    U32 v[3];    // (x, y) of each vertex as in the triangle header
    U32 lo, hi;  // box corners (lx, ly), (hx, hy)
    U32 entry;
    S32 who;     // threadIdx.x of the item's owner (warp * 32 + lane)
};

__device__ __forceinline__ U32 pack16(S32 a, S32 b) { return ((U32)a & 0xFFFFu) | ((U32)b << 16); }

struct RoundShared {
    BigItem big[kBinThreads];
    S32 numBig;
};

// Calls fn(cell, who, entry) for every cell touched by every valid item of
// the round. Items spanning at most kSmallCells cells are walked by their own
// thread; larger ones are dealt round-robin to the warps of the CTA and
// walked one cell per lane. Contains __syncthreads(); all threads must call it.
template <class Fn>
__device__ __forceinline__ void visitRound(RoundShared& rs, bool valid, const TriGeom& g, U32 entry, const Grid& gr,
                                           bool rebuild, Fn fn) {
    CellBox box{};
    int n = 0;
    if (valid) {
        box = cellBox(g, gr.halfW, gr.halfH, gr.cellLog2, gr.cx0, gr.cy0, gr.cx1, gr.cy1);
        n = box.count();
    }
    if (rebuild) {
        if (threadIdx.x == 0) rs.numBig = 0;
        __syncthreads();
        if (n > kSmallCells) {
            int k = atomicAdd(&rs.numBig, 1);
            BigItem& it = rs.big[k];
            it.v[0] = pack16(g.x0, g.y0);
            it.v[1] = pack16(g.x1, g.y1);
            it.v[2] = pack16(g.x2, g.y2);
            it.lo = pack16(box.lx, box.ly);
            it.hi = pack16(box.hx, box.hy);
            it.who = threadIdx.x;
            it.entry = entry;
        }
    }
    if (n > 0 && n <= kSmallCells) {
        for (S32 cy = box.ly; cy <= box.hy; cy++)
            for (S32 cx = box.lx; cx <= box.hx; cx++)
                if (cellTouched(g, box, cx, cy, gr.halfW, gr.halfH, gr.cellLog2)) fn(cellIndex(gr, cx, cy), (S32)threadIdx.x, entry);
    }
    __syncthreads();
    const int nb = rs.numBig;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int b = warp; b < nb; b += kBinWarps) {
        const BigItem& it = rs.big[b];
        const TriGeom bg = geomFromHeader(make_uint4(it.v[0], it.v[1], it.v[2], 0u));
        const CellBox bb{lo16(it.lo), hi16(it.lo), lo16(it.hi), hi16(it.hi)};
        const S32 who = it.who;
        const U32 e = it.entry;
        const S32 w = bb.hx - bb.lx + 1;
        const S32 cnt = bb.count();
        // Cell c of the box is (c % w, c / w); the quotient is taken in
        // binary32, exact here because c < 2^11 and w <= 2^5.
        const F32 invW = 1.0f / (F32)w;
        for (S32 c = lane; c < cnt; c += 32) {
            const S32 q = (S32)(((F32)c + 0.5f) * invW);
            const S32 cx = bb.lx + (c - q * w), cy = bb.ly + q;
            if (cellTouched(bg, bb, cx, cy, gr.halfW, gr.halfH, gr.cellLog2)) fn(cellIndex(gr, cx, cy), who, e);
        }
    }
}

__device__ __forceinline__ Grid binGrid(const InstanceDev* in, int binLog2) {
    Grid gr;
    gr.halfW = __ldg(&in->width) << (kSubpixelLog2 - 1);
    gr.halfH = __ldg(&in->height) << (kSubpixelLog2 - 1);
    gr.cellLog2 = binLog2 + kTileLog2 + kSubpixelLog2;
    gr.cx0 = 0;
    gr.cy0 = 0;
    gr.cx1 = __ldg(&in->widthBins) - 1;
    gr.cy1 = __ldg(&in->heightBins) - 1;
    gr.stride = __ldg(&in->widthBins);
    return gr;
}

// The chunk's subtriangle items stream through a window in shared memory
// (kWindow entries), so that every round holds up to kBinThreads live items:
// culled triangles carry none. Items keep (triangle, subtriangle) order.
constexpr int kWindow = kBinThreads * (kMaxSubtrisPerTri + 1);

// Appends the items of the next triangles of [next, t1) until the window
// holds at least kBinThreads items or the chunk is exhausted. Each thread
// takes kRefillTris consecutive triangles; if their items would overflow the
// window only the first kBinThreads triangles are taken (at most 7 items
// each, which always fit). fill and next are uniform across the CTA.
constexpr int kRefillTris = 4;

__device__ __forceinline__ S32 refillWindow(const DrawDev& d, S64& next, S64 t1, S32 fill, U32* s_items,
                                            S32* s_scratch) {
    __shared__ S32 s_cut;
    while (fill < kBinThreads && next < t1) {
        const S64 t = next + (S64)threadIdx.x * kRefillTris;
        int n[kRefillTris];
        int sum = 0;
#pragma unroll
        for (int j = 0; j < kRefillTris; j++) {
            n[j] = (t + j < t1) ? d.triSubtris[t + j] : 0;
            sum += n[j];
        }
        if (!__syncthreads_or(sum)) {
            next += kBinThreads * kRefillTris;
            continue;
        }
        S32 m;
        const S32 pos = blockExclusiveScan(sum, s_scratch, &m);
        // Items of the first kBinThreads triangles (threads below
        // kBinThreads / kRefillTris) end where the next thread's begin.
        if (threadIdx.x == kBinThreads / kRefillTris) s_cut = pos;
        __syncthreads();
        const bool all = fill + m <= kWindow;
        const bool take = all || (int)threadIdx.x < kBinThreads / kRefillTris;
        if (take) {
            S32 p = fill + pos;
#pragma unroll
            for (int j = 0; j < kRefillTris; j++)
                for (int s = 0; s < n[j]; s++) s_items[p++] = ((U32)(t + j) << 3) | (U32)(n[j] == 1 ? 7 : s);
        }
        fill += all ? m : s_cut;
        next += all ? (S64)kBinThreads * kRefillTris : (S64)kBinThreads;
        __syncthreads();
    }
    return fill;
}

// Drops the kBinThreads items of the round just processed from the window.
__device__ __forceinline__ S32 consumeWindow(U32* s_items, S32 fill) {
    const S32 rest = fill - kBinThreads;
    for (S32 i0 = 0; i0 < rest; i0 += kBinThreads) {
        const S32 i = i0 + threadIdx.x;
        const U32 v = (i < rest) ? s_items[kBinThreads + i] : 0u;
        __syncthreads();
        if (i < rest) s_items[i] = v;
        __syncthreads();
    }
    return rest > 0 ? rest : 0;
}

// ------------------------------------------------------------------ bin

// One CTA per chunk: counts the chunk's entries per bin.
__global__ void __launch_bounds__(kBinThreads, 2) binCountKernel(DrawDev d) {
    extern __shared__ S32 s_count[];
    __shared__ RoundShared rs;
    __shared__ U32 s_items[kWindow];
    __shared__ S32 s_scratch[kBinWarps + 1];
    __shared__ int s_inst;
    if (__ldg(&d.counters->overflow) & kOverflowSubtris) return;
    const int chunk = blockIdx.x;
    if (threadIdx.x == 0) s_inst = findInstance(d.chunkPrefix, d.numInstances, chunk);
    __syncthreads();
    const InstanceDev* in = &d.inst[s_inst];
    const Grid gr = binGrid(in, d.binLog2);
    const int nb = (gr.cx1 + 1) * (gr.cy1 + 1);
    for (int b = threadIdx.x; b < nb; b += kBinThreads) s_count[b] = 0;
    const int local = chunk - __ldg(&in->chunkBase);
    const S64 triBase = __ldg(&in->triBase);
    const S64 t0 = triBase + (S64)local * __ldg(&in->chunkTris);
    const S64 t1 = min(t0 + __ldg(&in->chunkTris), triBase + __ldg(&in->numTris));
    __syncthreads();
    S64 next = t0;
    for (S32 fill = 0;;) {
        fill = refillWindow(d, next, t1, fill, s_items, s_scratch);
        if (fill == 0) break;
        const bool valid = (S32)threadIdx.x < fill;
        TriGeom g{};
        U32 entry = 0;
        if (valid) {
            entry = s_items[threadIdx.x];
            g = geomFromHeader(d.triHeader[entrySlot(entry, d.triHeader)]);
        }
        visitRound(rs, valid, g, entry, gr, true, [&](int cell, S32, U32) { atomicAdd(&s_count[cell], 1); });
        __syncthreads();
        fill = consumeWindow(s_items, fill);
    }
    __syncthreads();
    S32* out = d.chunkBinCount + __ldg(&in->chunkCountBase) + (S64)local * nb;
    for (int b = threadIdx.x; b < nb; b += kBinThreads) out[b] = s_count[b];
}

// Run by the last bin-scan CTA to finish, once every bin's entry count is
// known: the coarse unit size (the caller's, or the smallest power of two
// from 64 that gives at most unitTarget units and fits maxUnits) and each
// bin's first unit. Contains barriers; the whole CTA calls it.
__device__ void planUnits(const DrawDev& d, S32* s_scratch) {
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
        const S32 n = b < d.totalBins ? (S32)(((S64)__ldcg(&d.binCount[b]) + U - 1) / U) : 0;
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
    S32* counts = d.chunkBinCount + __ldg(&in->chunkCountBase) + b;
    S32 carry = 0;
    for (int c0 = 0; c0 < nc; c0 += kBinThreads) {
        int c = c0 + threadIdx.x;
        S32 v = (c < nc) ? counts[(S64)c * nb] : 0;
        S32 tot;
        S32 ex = blockExclusiveScan(v, s_scratch, &tot);
        if (c < nc) counts[(S64)c * nb] = carry + ex;
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

// Per-cell scratch of a scatter CTA, carved from dynamic shared memory for
// ncells cells: per-warp ballot masks and prefixes, each cell's next free list
// index and round total, and the cells the current round touched (a bit per
// cell and a list), so the per-round bookkeeping costs O(touched cells).
struct ScatterSmem {
    U32* mask;     // [kBinWarps][ncells]
    S32* pre;      // [kBinWarps][ncells]
    S32* run;      // [ncells]
    S32* tot;      // [ncells]
    U32* touched;  // [(ncells + 31) / 32]
    S32* ntouch;   // [1]
    uint16_t* list;     // [ncells]
    int ncells;
};

__host__ __device__ inline size_t scatterSmemBytes(int ncells) {
    return sizeof(S32) * ((size_t)2 * kBinWarps * ncells + 2 * ncells + (ncells + 31) / 32 + 1) +
           sizeof(uint16_t) * (size_t)ncells;
}

__device__ __forceinline__ ScatterSmem carveScatter(S32* smem, int ncells) {
    ScatterSmem sm;
    sm.ncells = ncells;
    sm.mask = (U32*)smem;
    sm.pre = smem + kBinWarps * ncells;
    sm.run = sm.pre + kBinWarps * ncells;
    sm.tot = sm.run + ncells;
    sm.touched = (U32*)(sm.tot + ncells);
    sm.ntouch = (S32*)(sm.touched + (ncells + 31) / 32);
    sm.list = (uint16_t*)(sm.ntouch + 1);
    return sm;
}

// Zeroes masks and touch state (run is set by the caller). Ends with a barrier.
__device__ __forceinline__ void clearScatter(const ScatterSmem& sm) {
    for (int c = threadIdx.x; c < sm.ncells; c += kBinThreads)
        for (int w = 0; w < kBinWarps; w++) sm.mask[w * sm.ncells + c] = 0;
    for (int i = threadIdx.x; i < (sm.ncells + 31) / 32; i += kBinThreads) sm.touched[i] = 0;
    if (threadIdx.x == 0) *sm.ntouch = 0;
    __syncthreads();
}

// Ranked scatter of one round of items into per-cell lists: the rank of an
// entry in its cell is the number of earlier items (lower warp, then lower
// lane) of the round that touch the cell, plus the cell's running count.
// kTrack keeps the list of touched cells so the per-round bookkeeping costs
// O(touched cells) -- worth it over a bin grid, where a round touches few of
// up to 1024 bins; over the tiles of one bin most cells are touched and the
// dense loops are cheaper.
template <bool kTrack>
__device__ __forceinline__ void scatterRound(RoundShared& rs, bool valid, const TriGeom& g, U32 entry, const Grid& gr,
                                             const ScatterSmem& sm, U32* list, S64 capacity) {
    const int n = sm.ncells;
    visitRound(rs, valid, g, entry, gr, true, [&](int cell, S32 who, U32) {
        const U32 old = atomicOr(&sm.mask[(who >> 5) * n + cell], 1u << (who & 31));
        if (kTrack && old == 0u) {
            const U32 bit = 1u << (cell & 31);
            if (!(atomicOr(&sm.touched[cell >> 5], bit) & bit)) sm.list[atomicAdd(sm.ntouch, 1)] = (uint16_t)cell;
        }
    });
    __syncthreads();
    const int nt = kTrack ? *sm.ntouch : n;
    for (int i = threadIdx.x; i < nt; i += kBinThreads) {
        const int c = kTrack ? sm.list[i] : i;
        S32 acc = 0;
        for (int w = 0; w < kBinWarps; w++) {
            sm.pre[w * n + c] = acc;
            acc += __popc(sm.mask[w * n + c]);
        }
        sm.tot[c] = acc;
    }
    __syncthreads();
    visitRound(rs, valid, g, entry, gr, false, [&](int cell, S32 who, U32 e) {
        const int w = who >> 5;
        const U32 lt = (1u << (who & 31)) - 1u;
        S64 idx = (S64)sm.run[cell] + sm.pre[w * n + cell] + __popc(sm.mask[w * n + cell] & lt);
        if (idx < capacity) list[idx] = e;
    });
    __syncthreads();
    for (int i = threadIdx.x; i < nt; i += kBinThreads) {
        const int c = kTrack ? sm.list[i] : i;
        sm.run[c] += sm.tot[c];
        for (int w = 0; w < kBinWarps; w++) sm.mask[w * n + c] = 0;
        if (kTrack) sm.touched[c >> 5] = 0;
    }
    __syncthreads();
    if (kTrack && threadIdx.x == 0) *sm.ntouch = 0;
}

// One CTA per chunk: writes the chunk's entries into the bin lists. Within a
// round of up to 512 subtriangles the rank of an entry inside its bin is the
// number of earlier items (lower warp, then lower lane) that touch the same
// bin, taken from per-warp ballot masks.
__global__ void __launch_bounds__(kBinThreads, 2) binScatterKernel(DrawDev d) {
    extern __shared__ S32 smem[];
    __shared__ RoundShared rs;
    __shared__ U32 s_items[kWindow];
    __shared__ S32 s_scratch[kBinWarps + 1];
    __shared__ int s_inst;
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin)) return;
    const int chunk = blockIdx.x;
    if (threadIdx.x == 0) s_inst = findInstance(d.chunkPrefix, d.numInstances, chunk);
    __syncthreads();
    const InstanceDev* in = &d.inst[s_inst];
    const Grid gr = binGrid(in, d.binLog2);
    const int nb = (gr.cx1 + 1) * (gr.cy1 + 1);
    const ScatterSmem sm = carveScatter(smem, nb);
    clearScatter(sm);

    const int local = chunk - __ldg(&in->chunkBase);
    const S32 binBase = __ldg(&in->binBase);
    const S32* offs = d.chunkBinCount + __ldg(&in->chunkCountBase) + (S64)local * nb;
    for (int b = threadIdx.x; b < nb; b += kBinThreads) sm.run[b] = __ldg(&d.binStart[binBase + b]) + offs[b];
    const S64 triBase = __ldg(&in->triBase);
    const S64 t0 = triBase + (S64)local * __ldg(&in->chunkTris);
    const S64 t1 = min(t0 + __ldg(&in->chunkTris), triBase + __ldg(&in->numTris));
    __syncthreads();
    S64 next = t0;
    for (S32 fill = 0;;) {
        fill = refillWindow(d, next, t1, fill, s_items, s_scratch);
        if (fill == 0) break;
        const bool valid = (S32)threadIdx.x < fill;
        U32 entry = 0;
        TriGeom g{};
        if (valid) {
            entry = s_items[threadIdx.x];
            g = geomFromHeader(d.triHeader[entrySlot(entry, d.triHeader)]);
        }
        scatterRound<true>(rs, valid, g, entry, gr, sm, d.binList, d.maxBinEntries);
        fill = consumeWindow(s_items, fill);
    }
}

// --------------------------------------------------------------- coarse
//
// A coarse unit (up to unitEntries consecutive entries of one bin list) is
// taken by one warp, which walks it 32 entries (a group) at a time. A group is
// expanded into (entry, tile) pairs -- every tile of each entry's bounding
// box inside the bin -- and the pairs are dealt evenly over the lanes, so an
// entry covering many tiles costs its tile count / 32 iterations instead of
// holding up the whole warp. No CTA-wide barrier is involved: units, groups
// and ranks are all warp-local.

constexpr int kCoarseThreads = 256;
constexpr int kCoarseWarps = kCoarseThreads / 32;

// The current group of a warp, one word per entry (lane).
struct GroupSmem {
    S32 incl[32];   // inclusive prefix of the entries' box tile counts
    U32 v[3][32];   // vertices, packed as in the triangle header
    U32 box[32];    // lx | ly << 8 | w << 16 (bin-local tiles), bit 31: box of at most 2x2 tiles
    U32 mul[32];    // ceil(2^20 / w): tile k of the box is in row (k * mul) >> 20
    U32 entry[32];
};

// Loads the group's entries (lane i: list position e0 + i, valid below e1)
// and publishes them; returns the group's number of pairs.
__device__ __forceinline__ S32 stageGroup(const DrawDev& d, const Grid& gr, S32 e, S32 e1, GroupSmem& gs, S32& incl) {
    const int lane = threadIdx.x & 31;
    S32 n = 0;
    U32 entry = 0, box = 0, mul = 0;
    uint4 h = make_uint4(0u, 0u, 0u, 0u);
    if (e < e1) {
        entry = __ldg(&d.binList[e]);
        h = __ldg(&d.triHeader[entrySlot(entry, d.triHeader)]);
        const CellBox b = cellBox(geomFromHeader(h), gr.halfW, gr.halfH, gr.cellLog2, gr.cx0, gr.cy0, gr.cx1, gr.cy1);
        n = b.count();
        if (n > 0) {
            const U32 w = (U32)(b.hx - b.lx + 1);
            box = (U32)(b.lx - gr.cx0) | (U32)(b.ly - gr.cy0) << 8 | w << 16 | (b.small() ? 1u << 31 : 0u);
            mul = ((1u << 20) + w - 1u) / w;
        }
    }
    incl = warpInclusiveScan(n);
    gs.incl[lane] = incl;
    gs.v[0][lane] = h.x;
    gs.v[1][lane] = h.y;
    gs.v[2][lane] = h.z;
    gs.box[lane] = box;
    gs.mul[lane] = mul;
    gs.entry[lane] = entry;
    __syncwarp();
    return __shfl_sync(0xFFFFFFFFu, incl, 31);
}

// Pair p of the group (p below the group's pair count): its entry j and its
// bin-local cell; returns whether the entry's triangle may touch the tile.
// The quotient k / w is exact for k < 2^10 and w <= 32 (error below 2^-10).
__device__ __forceinline__ bool pairCell(const GroupSmem& gs, const Grid& gr, S32 p, int& j, int& cell) {
    int jj = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1)
        if (gs.incl[jj + s - 1] <= p) jj += s;
    const S32 k = p - (jj ? gs.incl[jj - 1] : 0);
    const U32 box = gs.box[jj];
    const S32 w = (S32)((box >> 16) & 0xFFu);
    const S32 q = (S32)(((U32)k * gs.mul[jj]) >> 20);
    const S32 lx = (S32)(box & 0xFFu) + k - q * w;
    const S32 ly = (S32)((box >> 8) & 0xFFu) + q;
    j = jj;
    cell = ly * gr.stride + lx;
    if (box >> 31) return true;
    const TriGeom g = geomFromHeader(make_uint4(gs.v[0][jj], gs.v[1][jj], gs.v[2][jj], 0u));
    const S32 side = 1 << gr.cellLog2;
    const S32 rx0 = ((gr.cx0 + lx) << gr.cellLog2) - gr.halfW, ry0 = ((gr.cy0 + ly) << gr.cellLog2) - gr.halfH;
    return triTouchesRect(g, rx0, ry0, rx0 + side - 1, ry0 + side - 1);
}

struct UnitInfo {
    const InstanceDev* in;
    S32 gb, seg, bx, by, e0, e1;
};

// Next coarse unit for this warp (dynamic assignment); uniform across the warp.
__device__ __forceinline__ int warpNextUnit(S32* counter) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(counter, 1);
    return __shfl_sync(0xFFFFFFFFu, u, 0);
}

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
    gr.cx0 = ui.bx << binLog2;
    gr.cy0 = ui.by << binLog2;
    gr.cx1 = min(gr.cx0 + side - 1, __ldg(&ui.in->widthTiles) - 1);
    gr.cy1 = min(gr.cy0 + side - 1, __ldg(&ui.in->heightTiles) - 1);
    gr.stride = side;
    return gr;
}

// Persistent warps over coarse units (taken dynamically): per-unit tile counts.
__global__ void __launch_bounds__(kCoarseThreads) coarseCountKernel(DrawDev d) {
    extern __shared__ S32 smem[];
    __shared__ GroupSmem s_group[kCoarseWarps];
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tpb = 1 << (2 * d.binLog2);
    S32* cnt = smem + warp * tpb;
    GroupSmem& gs = s_group[warp];
    const S32 numUnits = (S32)min((S64)__ldg(&d.counters->numUnits), d.maxUnits);
    const S32 unitEntries = __ldg(&d.counters->unitEntries);
    for (;;) {
        const int u = warpNextUnit(&d.counters->coarseWork[0]);
        if (u >= numUnits) break;
        UnitInfo ui;
        loadUnit(d, u, unitEntries, ui);
        const Grid gr = tileGrid(ui, d.binLog2);
        for (int t = lane; t < tpb; t += 32) cnt[t] = 0;
        __syncwarp();
        for (S32 e0 = ui.e0; e0 < ui.e1; e0 += 32) {
            S32 incl;
            const S32 P = stageGroup(d, gr, e0 + lane, ui.e1, gs, incl);
            for (S32 p = lane; p < P; p += 32) {
                int j, cell;
                if (pairCell(gs, gr, p, j, cell)) atomicAdd(&cnt[cell], 1);
            }
            __syncwarp();
        }
        S32* out = d.unitTileCount + (S64)u * tpb;
        for (int t = lane; t < tpb; t += 32) out[t] = cnt[t];
        __syncwarp();
    }
}

// One CTA per global bin: unit-order offsets per tile, tile list allocation.
__global__ void __launch_bounds__(kBinThreads) coarseScanKernel(DrawDev d) {
    __shared__ S32 s_scratch[kBinWarps + 1];
    __shared__ int s_inst;
    __shared__ S32 s_base;
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin)) return;
    const int gb = blockIdx.x;
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
    const S32 first = __ldg(&d.binUnitFirst[gb]);
    S32 carry = 0;
    for (int t0 = 0; t0 < tpb; t0 += kBinThreads) {
        int t = t0 + threadIdx.x;
        S32 acc = 0;
        if (t < tpb) {
            S32* col = d.unitTileCount + (S64)first * tpb + t;
            // Eight units per step: the loads are issued before the stores.
            S32 k = 0;
            for (; k + 8 <= units; k += 8) {
                S32 c[8];
#pragma unroll
                for (int i = 0; i < 8; i++) c[i] = col[(S64)(k + i) * tpb];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    col[(S64)(k + i) * tpb] = acc;
                    acc += c[i];
                }
            }
            for (; k < units; k++) {
                const S32 c = col[(S64)k * tpb];
                col[(S64)k * tpb] = acc;
                acc += c;
            }
        }
        S32 tot;
        S32 ex = blockExclusiveScan(acc, s_scratch, &tot);
        if (t < tpb) {
            S32 tx = (bx << d.binLog2) + (t & (side - 1));
            S32 ty = (by << d.binLog2) + (t >> d.binLog2);
            if (tx < wt && ty < ht) {
                S32 gt = tileBase + ty * wt + tx;
                d.tileCount[gt] = acc;
                d.tileStart[gt] = carry + ex;   // relative; rebased below
            }
        }
        carry += tot;
    }
    if (threadIdx.x == 0) {
        S32 base = atomicAdd(&d.counters->tileEntries, carry);
        if ((S64)base + carry > d.maxTileEntries) atomicOr(&d.counters->overflow, kOverflowTile);
        s_base = base;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < tpb; t += kBinThreads) {
        S32 tx = (bx << d.binLog2) + (t & (side - 1));
        S32 ty = (by << d.binLog2) + (t >> d.binLog2);
        if (tx < wt && ty < ht) d.tileStart[tileBase + ty * wt + tx] += s_base;
    }
}

// Persistent warps over coarse units (taken dynamically): writes tile list
// entries. Within a group the rank of an entry in a tile list is the number of
// earlier entries of the group touching the tile (a per-tile mask, one bit per
// entry) plus the tile's running index. A group whose pairs exceed the per-
// warp hit buffer (one slot per tile of the bin) is taken in sub-groups that
// end at entry boundaries; one entry never has more pairs than the bin has
// tiles.
__global__ void __launch_bounds__(kCoarseThreads) coarseScatterKernel(DrawDev d) {
    extern __shared__ S32 smem[];
    __shared__ GroupSmem s_group[kCoarseWarps];
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin | kOverflowTile)) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const U32 ltMask = (1u << lane) - 1u;
    const int tpb = 1 << (2 * d.binLog2);
    const S32 side = 1 << d.binLog2;
    U32* mask = (U32*)smem + (size_t)warp * 3 * tpb;   // [tpb] entries of the sub-group per tile
    S32* run = (S32*)(mask + tpb);                      // [tpb] next free list index per tile
    U32* hits = (U32*)(run + tpb);                      // [tpb] cell | entry << 16 of touching pairs
    GroupSmem& gs = s_group[warp];
    for (int t = lane; t < tpb; t += 32) mask[t] = 0u;
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
        for (S32 e0 = ui.e0; e0 < ui.e1; e0 += 32) {
            S32 incl;
            const S32 P = stageGroup(d, gr, e0 + lane, ui.e1, gs, incl);
            for (S32 p0 = 0; p0 < P;) {
                // Entries whose pairs all lie below p0 + tpb form the sub-group.
                const int jEnd = __popc(__ballot_sync(0xFFFFFFFFu, incl <= p0 + tpb));
                const S32 p1 = __shfl_sync(0xFFFFFFFFu, incl, jEnd - 1);
                S32 nh = 0;
                for (S32 base = p0; base < p1; base += 32) {
                    const S32 p = base + lane;
                    int j = 0, cell = 0;
                    const bool hit = p < p1 && pairCell(gs, gr, p, j, cell);
                    if (hit) atomicOr(&mask[cell], 1u << j);
                    const U32 b = __ballot_sync(0xFFFFFFFFu, hit);
                    if (hit) hits[nh + __popc(b & ltMask)] = (U32)cell | (U32)j << 16;
                    nh += __popc(b);
                }
                __syncwarp();
                for (S32 h = lane; h < nh; h += 32) {
                    const U32 hc = hits[h];
                    const int cell = (int)(hc & 0xFFFFu), j = (int)(hc >> 16);
                    const S64 idx = (S64)run[cell] + __popc(mask[cell] & ((1u << j) - 1u));
                    if (idx < d.maxTileEntries) d.tileList[idx] = gs.entry[j];
                }
                __syncwarp();
                // The last entry of the sub-group touching a tile advances the
                // tile's index and clears its mask.
                for (S32 h = lane; h < nh; h += 32) {
                    const U32 hc = hits[h];
                    const int cell = (int)(hc & 0xFFFFu), j = (int)(hc >> 16);
                    const U32 m = mask[cell];
                    if ((m >> j) == 1u) {
                        run[cell] += __popc(m);
                        mask[cell] = 0u;
                    }
                }
                __syncwarp();
                p0 = p1;
            }
        }
    }
}

// ------------------------------------------------------------ launchers

size_t binScatterSmem(int maxBins) { return scatterSmemBytes(maxBins); }
size_t coarseCountSmem(int binLog2) { return sizeof(S32) * kCoarseWarps * ((size_t)1 << (2 * binLog2)); }
size_t coarseScatterSmem(int binLog2) { return sizeof(S32) * 3 * kCoarseWarps * ((size_t)1 << (2 * binLog2)); }

cudaError_t launchBinning(const DrawDev& d, int maxBins, int numSMs, cudaStream_t stream, cudaEvent_t evCoarse) {
    // Resident coarse CTAs per SM for bins of 8, 16 and 32 tiles a side.
    static int coarseCountCtas[6] = {}, coarseScatterCtas[6] = {};
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(binScatterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        cudaFuncSetAttribute(coarseScatterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        cudaFuncSetAttribute(binCountKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        cudaFuncSetAttribute(coarseCountKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        for (int b = 3; b <= 5; b++) {
            int n = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, coarseCountKernel, kCoarseThreads, coarseCountSmem(b));
            coarseCountCtas[b] = n > 0 ? n : 1;
            n = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, coarseScatterKernel, kCoarseThreads, coarseScatterSmem(b));
            coarseScatterCtas[b] = n > 0 ? n : 1;
        }
        configured = true;
    }
    const int bl = d.binLog2 >= 3 && d.binLog2 <= 5 ? d.binLog2 : 4;
    // Units sized on the device: about two per resident coarse-scatter warp.
    DrawDev dl = d;
    dl.unitTarget = 2 * numSMs * coarseScatterCtas[bl] * kCoarseWarps;
    // binScan also runs for a draw without triangles: it zeroes the bin counts.
    if (dl.totalChunks > 0) binCountKernel<<<dl.totalChunks, kBinThreads, sizeof(S32) * maxBins, stream>>>(dl);
    binScanKernel<<<dl.totalBins, kBinThreads, 0, stream>>>(dl);
    if (dl.totalChunks > 0) binScatterKernel<<<dl.totalChunks, kBinThreads, binScatterSmem(maxBins), stream>>>(dl);
    if (evCoarse) cudaEventRecord(evCoarse, stream);
    // Persistent coarse warps: as many CTAs as are resident at once, and no
    // more than the draw's units can keep busy.
    const S64 unitCtas = (dl.maxUnits + kCoarseWarps - 1) / kCoarseWarps;
    const int countGrid = (int)min((S64)numSMs * coarseCountCtas[bl], unitCtas);
    const int scatterGrid = (int)min((S64)numSMs * coarseScatterCtas[bl], unitCtas);
    coarseCountKernel<<<countGrid, kCoarseThreads, coarseCountSmem(dl.binLog2), stream>>>(dl);
    coarseScanKernel<<<dl.totalBins, kBinThreads, 0, stream>>>(dl);
    coarseScatterKernel<<<scatterGrid, kCoarseThreads, coarseScatterSmem(dl.binLog2), stream>>>(dl);
    return cudaGetLastError();
}

}  // namespace cr
