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
//   coarse: units of consecutive bin-list entries of one bin, with the same
//           three passes over the tiles of the bin.
//
// In every round, an item whose bounding box spans more than kSmallCells
// cells is dealt to a warp (one cell per lane) instead of being walked by its
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

// Items too large for their own thread, walked by a whole warp.
struct BigItem {
    TriGeom g;
    CellBox box;
    S32 who;     // threadIdx.x of the item's owner (warp * 32 + lane)
    U32 entry;
};

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
            rs.big[k].g = g;
            rs.big[k].box = box;
            rs.big[k].who = threadIdx.x;
            rs.big[k].entry = entry;
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
        const S32 w = it.box.hx - it.box.lx + 1;
        const S32 cnt = it.box.count();
        // Cell c of the box is (c % w, c / w); the quotient is taken in
        // binary32, exact here because c < 2^11 and w <= 2^5.
        const F32 invW = 1.0f / (F32)w;
        for (S32 c = lane; c < cnt; c += 32) {
            const S32 q = (S32)(((F32)c + 0.5f) * invW);
            const S32 cx = it.box.lx + (c - q * w), cy = it.box.ly + q;
            if (cellTouched(it.g, it.box, cx, cy, gr.halfW, gr.halfH, gr.cellLog2)) fn(cellIndex(gr, cx, cy), it.who, it.entry);
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

// Items of a bin-stage round: triangles [r0, r0 + 512) of the chunk expanded
// into their subtriangles, in (triangle, subtriangle) order.
struct ItemRound {
    S32 m;  // number of items
};

__device__ __forceinline__ ItemRound expandRound(const DrawDev& d, S64 r0, S64 t1, U32* s_items, S32* s_scratch) {
    S64 t = r0 + threadIdx.x;
    int n = (t < t1) ? d.triSubtris[t] : 0;
    S32 m;
    S32 pos = blockExclusiveScan(n, s_scratch, &m);
    for (int s = 0; s < n; s++) s_items[pos + s] = ((U32)t << 3) | (U32)(n == 1 ? 7 : s);
    __syncthreads();
    return ItemRound{m};
}

// ------------------------------------------------------------------ bin

// One CTA per chunk: counts the chunk's entries per bin.
__global__ void __launch_bounds__(kBinThreads, 2) binCountKernel(DrawDev d) {
    extern __shared__ S32 s_count[];
    __shared__ RoundShared rs;
    __shared__ U32 s_items[kBinThreads * kMaxSubtrisPerTri];
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
    for (S64 r0 = t0; r0 < t1; r0 += kBinThreads) {
        ItemRound ir = expandRound(d, r0, t1, s_items, s_scratch);
        for (S32 k0 = 0; k0 < ir.m; k0 += kBinThreads) {
            const S32 k = k0 + threadIdx.x;
            const bool valid = k < ir.m;
            TriGeom g{};
            U32 entry = 0;
            if (valid) {
                entry = s_items[k];
                g = geomFromHeader(d.triHeader[entrySlot(entry, d.triHeader)]);
            }
            visitRound(rs, valid, g, entry, gr, true, [&](int cell, S32, U32) { atomicAdd(&s_count[cell], 1); });
            __syncthreads();
        }
    }
    __syncthreads();
    S32* out = d.chunkBinCount + __ldg(&in->chunkCountBase) + (S64)local * nb;
    for (int b = threadIdx.x; b < nb; b += kBinThreads) out[b] = s_count[b];
}

// One CTA per global bin: chunk-order exclusive offsets, list allocation and
// coarse work units.
__global__ void __launch_bounds__(kBinThreads) binScanKernel(DrawDev d) {
    __shared__ S32 s_scratch[kBinWarps + 1];
    __shared__ int s_inst;
    __shared__ S32 s_units, s_unitFirst;
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
        S32 units = (carry + d.unitEntries - 1) / d.unitEntries;
        S32 first = atomicAdd(&d.counters->numUnits, units);
        d.binUnitFirst[gb] = first;
        s_units = units;
        s_unitFirst = first;
    }
    __syncthreads();
    const S32 units = s_units, first = s_unitFirst;
    for (int k = threadIdx.x; k < units; k += kBinThreads) {
        if ((S64)first + k < d.maxUnits) {
            d.unitBin[first + k] = gb;
            d.unitSeg[first + k] = k;
        }
    }
}

// Ranked scatter of one round of items into per-cell lists. s_mask/s_pre are
// [kBinWarps][ncells]; s_run holds each cell's next free list index.
__device__ __forceinline__ void scatterRound(RoundShared& rs, bool valid, const TriGeom& g, U32 entry, const Grid& gr,
                                             int ncells, U32* s_mask, S32* s_pre, S32* s_run, S32* s_tot, U32* list,
                                             S64 capacity) {
    visitRound(rs, valid, g, entry, gr, true, [&](int cell, S32 who, U32) {
        atomicOr(&s_mask[(who >> 5) * ncells + cell], 1u << (who & 31));
    });
    __syncthreads();
    for (int c = threadIdx.x; c < ncells; c += kBinThreads) {
        S32 acc = 0;
        for (int w = 0; w < kBinWarps; w++) {
            s_pre[w * ncells + c] = acc;
            acc += __popc(s_mask[w * ncells + c]);
        }
        s_tot[c] = acc;
    }
    __syncthreads();
    visitRound(rs, valid, g, entry, gr, false, [&](int cell, S32 who, U32 e) {
        const int w = who >> 5;
        const U32 lt = (1u << (who & 31)) - 1u;
        S64 idx = (S64)s_run[cell] + s_pre[w * ncells + cell] + __popc(s_mask[w * ncells + cell] & lt);
        if (idx < capacity) list[idx] = e;
    });
    __syncthreads();
    for (int c = threadIdx.x; c < ncells; c += kBinThreads) {
        s_run[c] += s_tot[c];
        for (int w = 0; w < kBinWarps; w++) s_mask[w * ncells + c] = 0;
    }
    __syncthreads();
}

// One CTA per chunk: writes the chunk's entries into the bin lists. Within a
// round of up to 512 subtriangles the rank of an entry inside its bin is the
// number of earlier items (lower warp, then lower lane) that touch the same
// bin, taken from per-warp ballot masks.
__global__ void __launch_bounds__(kBinThreads, 2) binScatterKernel(DrawDev d) {
    extern __shared__ S32 smem[];
    __shared__ RoundShared rs;
    __shared__ U32 s_items[kBinThreads * kMaxSubtrisPerTri];
    __shared__ S32 s_scratch[kBinWarps + 1];
    __shared__ int s_inst;
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin)) return;
    const int chunk = blockIdx.x;
    if (threadIdx.x == 0) s_inst = findInstance(d.chunkPrefix, d.numInstances, chunk);
    __syncthreads();
    const InstanceDev* in = &d.inst[s_inst];
    const Grid gr = binGrid(in, d.binLog2);
    const int nb = (gr.cx1 + 1) * (gr.cy1 + 1);
    U32* s_mask = (U32*)smem;                         // [kBinWarps][nb]
    S32* s_pre = smem + kBinWarps * nb;               // [kBinWarps][nb]
    S32* s_run = s_pre + kBinWarps * nb;              // [nb]
    S32* s_tot = s_run + nb;                          // [nb]

    const int local = chunk - __ldg(&in->chunkBase);
    const S32 binBase = __ldg(&in->binBase);
    const S32* offs = d.chunkBinCount + __ldg(&in->chunkCountBase) + (S64)local * nb;
    for (int b = threadIdx.x; b < nb; b += kBinThreads) {
        s_run[b] = __ldg(&d.binStart[binBase + b]) + offs[b];
        for (int w = 0; w < kBinWarps; w++) s_mask[w * nb + b] = 0;
    }
    const S64 triBase = __ldg(&in->triBase);
    const S64 t0 = triBase + (S64)local * __ldg(&in->chunkTris);
    const S64 t1 = min(t0 + __ldg(&in->chunkTris), triBase + __ldg(&in->numTris));
    __syncthreads();
    for (S64 r0 = t0; r0 < t1; r0 += kBinThreads) {
        ItemRound ir = expandRound(d, r0, t1, s_items, s_scratch);
        for (S32 k0 = 0; k0 < ir.m; k0 += kBinThreads) {
            const S32 k = k0 + threadIdx.x;
            const bool valid = k < ir.m;
            U32 entry = 0;
            TriGeom g{};
            if (valid) {
                entry = s_items[k];
                g = geomFromHeader(d.triHeader[entrySlot(entry, d.triHeader)]);
            }
            scatterRound(rs, valid, g, entry, gr, nb, s_mask, s_pre, s_run, s_tot, d.binList, d.maxBinEntries);
        }
    }
}

// --------------------------------------------------------------- coarse

struct UnitInfo {
    const InstanceDev* in;
    S32 gb, seg, bx, by, e0, e1;
};

__device__ __forceinline__ void loadUnit(const DrawDev& d, int u, UnitInfo& ui, int* s_inst) {
    if (threadIdx.x == 0) *s_inst = findInstance(d.binPrefix, d.numInstances, __ldg(&d.unitBin[u]));
    __syncthreads();
    ui.in = &d.inst[*s_inst];
    ui.gb = __ldg(&d.unitBin[u]);
    ui.seg = __ldg(&d.unitSeg[u]);
    S32 b = ui.gb - __ldg(&ui.in->binBase);
    S32 wb = __ldg(&ui.in->widthBins);
    ui.bx = b % wb;
    ui.by = b / wb;
    S32 start = __ldg(&d.binStart[ui.gb]), cnt = __ldg(&d.binCount[ui.gb]);
    ui.e0 = start + ui.seg * d.unitEntries;
    ui.e1 = min(ui.e0 + d.unitEntries, start + cnt);
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

// Persistent CTAs over coarse units: per-unit tile counts.
__global__ void __launch_bounds__(kBinThreads, 2) coarseCountKernel(DrawDev d) {
    extern __shared__ S32 s_count[];
    __shared__ RoundShared rs;
    __shared__ int s_inst;
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin)) return;
    const int tpb = 1 << (2 * d.binLog2);
    const S32 numUnits = (S32)min((S64)*(volatile S32*)&d.counters->numUnits, d.maxUnits);
    for (int u = blockIdx.x; u < numUnits; u += gridDim.x) {
        UnitInfo ui;
        loadUnit(d, u, ui, &s_inst);
        for (int t = threadIdx.x; t < tpb; t += kBinThreads) s_count[t] = 0;
        const Grid gr = tileGrid(ui, d.binLog2);
        __syncthreads();
        for (S32 e0 = ui.e0; e0 < ui.e1; e0 += kBinThreads) {
            const S32 e = e0 + threadIdx.x;
            const bool valid = e < ui.e1;
            U32 entry = 0;
            TriGeom g{};
            if (valid) {
                entry = __ldg(&d.binList[e]);
                g = geomFromHeader(d.triHeader[entrySlot(entry, d.triHeader)]);
            }
            visitRound(rs, valid, g, entry, gr, true, [&](int cell, S32, U32) { atomicAdd(&s_count[cell], 1); });
            __syncthreads();
        }
        for (int t = threadIdx.x; t < tpb; t += kBinThreads) d.unitTileCount[(S64)u * tpb + t] = s_count[t];
        __syncthreads();
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
    const S32 units = (cnt + d.unitEntries - 1) / d.unitEntries;
    const S32 first = __ldg(&d.binUnitFirst[gb]);
    S32 carry = 0;
    for (int t0 = 0; t0 < tpb; t0 += kBinThreads) {
        int t = t0 + threadIdx.x;
        S32 acc = 0;
        if (t < tpb) {
            for (S32 k = 0; k < units; k++) {
                S32* p = &d.unitTileCount[(S64)(first + k) * tpb + t];
                S32 c = *p;
                *p = acc;
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

// Persistent CTAs over coarse units: writes tile list entries, ranked per
// 512-entry round by per-warp ballot masks over the tiles of the bin.
__global__ void __launch_bounds__(kBinThreads, 2) coarseScatterKernel(DrawDev d) {
    extern __shared__ S32 smem[];
    __shared__ RoundShared rs;
    __shared__ int s_inst;
    if (__ldg(&d.counters->overflow) & (kOverflowSubtris | kOverflowBin | kOverflowTile)) return;
    const int tpb = 1 << (2 * d.binLog2);
    const S32 side = 1 << d.binLog2;
    U32* s_mask = (U32*)smem;                // [kBinWarps][tpb]
    S32* s_pre = smem + kBinWarps * tpb;     // [kBinWarps][tpb]
    S32* s_run = s_pre + kBinWarps * tpb;    // [tpb]
    S32* s_tot = s_run + tpb;                // [tpb]
    const S32 numUnits = (S32)min((S64)*(volatile S32*)&d.counters->numUnits, d.maxUnits);
    for (int t = threadIdx.x; t < tpb; t += kBinThreads)
        for (int w = 0; w < kBinWarps; w++) s_mask[w * tpb + t] = 0;
    for (int u = blockIdx.x; u < numUnits; u += gridDim.x) {
        UnitInfo ui;
        loadUnit(d, u, ui, &s_inst);
        const Grid gr = tileGrid(ui, d.binLog2);
        const S32 wt = __ldg(&ui.in->widthTiles);
        const S32 tileBase = __ldg(&ui.in->tileBase);
        for (int t = threadIdx.x; t < tpb; t += kBinThreads) {
            S32 tx = gr.cx0 + (t & (side - 1)), ty = gr.cy0 + (t >> d.binLog2);
            S32 v = 0;
            if (tx <= gr.cx1 && ty <= gr.cy1)
                v = __ldg(&d.tileStart[tileBase + ty * wt + tx]) + __ldg(&d.unitTileCount[(S64)u * tpb + t]);
            s_run[t] = v;
        }
        __syncthreads();
        for (S32 e0 = ui.e0; e0 < ui.e1; e0 += kBinThreads) {
            const S32 e = e0 + threadIdx.x;
            const bool valid = e < ui.e1;
            U32 entry = 0;
            TriGeom g{};
            if (valid) {
                entry = __ldg(&d.binList[e]);
                g = geomFromHeader(d.triHeader[entrySlot(entry, d.triHeader)]);
            }
            scatterRound(rs, valid, g, entry, gr, tpb, s_mask, s_pre, s_run, s_tot, d.tileList, d.maxTileEntries);
        }
    }
}

// ------------------------------------------------------------ launchers

size_t binScatterSmem(int maxBins) {
    return sizeof(S32) * ((size_t)2 * kBinWarps * maxBins + 2 * maxBins);
}
size_t coarseScatterSmem(int binLog2) {
    int tpb = 1 << (2 * binLog2);
    return sizeof(S32) * ((size_t)2 * kBinWarps * tpb + 2 * tpb);
}

cudaError_t launchBinning(const DrawDev& d, int maxBins, int numSMs, cudaStream_t stream, cudaEvent_t evCoarse) {
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(binScatterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        cudaFuncSetAttribute(coarseScatterKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        cudaFuncSetAttribute(binCountKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        cudaFuncSetAttribute(coarseCountKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
        configured = true;
    }
    const int tpb = 1 << (2 * d.binLog2);
    // binScan also runs for a draw without triangles: it zeroes the bin counts.
    if (d.totalChunks > 0) binCountKernel<<<d.totalChunks, kBinThreads, sizeof(S32) * maxBins, stream>>>(d);
    binScanKernel<<<d.totalBins, kBinThreads, 0, stream>>>(d);
    if (d.totalChunks > 0) binScatterKernel<<<d.totalChunks, kBinThreads, binScatterSmem(maxBins), stream>>>(d);
    if (evCoarse) cudaEventRecord(evCoarse, stream);
    const int coarseGrid = numSMs * 3;
    coarseCountKernel<<<coarseGrid, kBinThreads, sizeof(S32) * tpb, stream>>>(d);
    coarseScanKernel<<<d.totalBins, kBinThreads, 0, stream>>>(d);
    coarseScatterKernel<<<coarseGrid, kBinThreads, coarseScatterSmem(d.binLog2), stream>>>(d);
    return cudaGetLastError();
}

}  // namespace cr
