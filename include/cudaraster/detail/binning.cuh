// binning.cuh -- conservative triangle-vs-rectangle tests shared by the bin
// and coarse stages. A triangle is kept for a bin / tile unless its bounding
// box (at one sample per pixel: the box of the pixel centres inside it) misses
// it or one edge has the whole rectangle strictly outside; exact
// per-sample coverage is decided later by the fine stage, so a kept triangle
// that covers no sample changes no output bit. The reference makes the same
// conservative choice with its bbox fast paths and corner tests
// (BinRaster.inl:208-300, CoarseRaster.inl:299-435).
#pragma once

#include "device.cuh"

namespace cr {

struct TriGeom {
    S32 x0, y0, x1, y1, x2, y2;   // header frame: subpixels relative to the viewport centre
};

__device__ __forceinline__ TriGeom geomFromHeader(uint4 h) {
    TriGeom g;
    g.x0 = lo16(h.x); g.y0 = hi16(h.x);
    g.x1 = lo16(h.y); g.y1 = hi16(h.y);
    g.x2 = lo16(h.z); g.y2 = hi16(h.z);
    return g;
}

// max over the closed rectangle [rx0, rx1] x [ry0, ry1] of (o - P) x d,
// compared against zero: returns false if the rectangle lies strictly on the
// outer side of the edge line.
__device__ __forceinline__ bool edgeTouchesRect(S32 ox, S32 oy, S32 dx, S32 dy, S32 rx0, S32 ry0, S32 rx1, S32 ry1) {
    S32 px = dy > 0 ? rx0 : rx1;
    S32 py = dx > 0 ? ry1 : ry0;
    S64 e = (S64)(ox - px) * dy - (S64)(oy - py) * dx;
    return e >= 0;
}

__device__ __forceinline__ bool triTouchesRect(const TriGeom& g, S32 rx0, S32 ry0, S32 rx1, S32 ry1) {
    return edgeTouchesRect(g.x0, g.y0, g.x1 - g.x0, g.y1 - g.y0, rx0, ry0, rx1, ry1) &&
           edgeTouchesRect(g.x1, g.y1, g.x2 - g.x1, g.y2 - g.y1, rx0, ry0, rx1, ry1) &&
           edgeTouchesRect(g.x2, g.y2, g.x0 - g.x2, g.y0 - g.y2, rx0, ry0, rx1, ry1);
}

// Cell range of a triangle's bounding box, clamped to [cx0, cx1] x [cy0, cy1].
struct CellBox {
    S32 lx, ly, hx, hy;
    __device__ __forceinline__ S32 count() const { return (lx > hx || ly > hy) ? 0 : (hx - lx + 1) * (hy - ly + 1); }
    __device__ __forceinline__ bool small() const { return (hx - lx) <= 1 && (hy - ly) <= 1; }
};

// With one sample per pixel (centerOnly) the box is that of the pixel centres
// inside the vertex box: pixel p's centre lies at 16 p + 8 subpixels from the
// viewport's left edge, so the first centre at or right of x is pixel
// (x + 7) >> 4 and the last at or left of x is (x - 8) >> 4 (x from that edge);
// a cell whose pixel centres all miss the vertex box holds no sample the fine
// stage could cover. With MSAA the samples spread over the pixel, and the box
// is that of the vertices.
__device__ __forceinline__ CellBox cellBox(const TriGeom& g, S32 halfW, S32 halfH, int cellLog2,
                                           S32 cx0, S32 cy0, S32 cx1, S32 cy1, bool centerOnly) {
    const S32 lo = centerOnly ? 7 : 0, hi = centerOnly ? 8 : 0;
    CellBox b;
    b.lx = max((min3i(g.x0, g.x1, g.x2) + halfW + lo) >> cellLog2, cx0);
    b.hx = min((max3i(g.x0, g.x1, g.x2) + halfW - hi) >> cellLog2, cx1);
    b.ly = max((min3i(g.y0, g.y1, g.y2) + halfH + lo) >> cellLog2, cy0);
    b.hy = min((max3i(g.y0, g.y1, g.y2) + halfH - hi) >> cellLog2, cy1);
    return b;
}

// List entry <-> data slot: entry = triangle << 3 | subtriangle, 7 = the
// triangle's own slot (BinRaster.inl:148-158).
__device__ __forceinline__ S64 entrySlot(U32 entry, const uint4* triHeader) {
    U32 tri = entry >> 3, sub = entry & 7;
    if (sub == 7) return (S64)tri;
    return (S64)__ldg(&triHeader[tri].w) + sub;
}

// Warp-level inclusive scan.
__device__ __forceinline__ S32 warpInclusiveScan(S32 v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        S32 t = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

}  // namespace cr
