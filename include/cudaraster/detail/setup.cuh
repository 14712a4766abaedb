// setup.cuh -- triangle setup kernel (stage 1 of 4).
//
// Restates TriangleSetup.inl:19-417 of the reference for sm_103a: one thread
// per input triangle; frustum cull, snap to the 1/16-px grid, backface /
// between-samples cull, clip-path subtriangles, depth and barycentric plane
// equations, edge flip bits. Differences from the reference are structural
// only: vertices are read with __ldg instead of a legacy texture reference,
// several scenes share one launch (per-instance descriptors), and extra
// subtriangle slots are allocated from a counter past all triangle slots.
#pragma once

#include "device.cuh"
#include "launch.h"

namespace cr {

struct SnapOut {
    int2 p0, p1, p2, lo, hi;
    F32 rcpW0, rcpW1, rcpW2;
};

// snapTriangle (TriangleSetup.inl:19-31)
__device__ __forceinline__ SnapOut snapTriangle(float4 v0, float4 v1, float4 v2, S32 width, S32 height) {
    SnapOut o;
    F32 sx = (F32)(width << (kSubpixelLog2 - 1));
    F32 sy = (F32)(height << (kSubpixelLog2 - 1));
    o.rcpW0 = frcp(v0.w);
    o.rcpW1 = frcp(v1.w);
    o.rcpW2 = frcp(v2.w);
    o.p0 = make_int2(f32_to_s32_sat(fmul(fmul(v0.x, o.rcpW0), sx)), f32_to_s32_sat(fmul(fmul(v0.y, o.rcpW0), sy)));
    o.p1 = make_int2(f32_to_s32_sat(fmul(fmul(v1.x, o.rcpW1), sx)), f32_to_s32_sat(fmul(fmul(v1.y, o.rcpW1), sy)));
    o.p2 = make_int2(f32_to_s32_sat(fmul(fmul(v2.x, o.rcpW2), sx)), f32_to_s32_sat(fmul(fmul(v2.y, o.rcpW2), sy)));
    o.lo = make_int2(min3i(o.p0.x, o.p1.x, o.p2.x), min3i(o.p0.y, o.p1.y, o.p2.y));
    o.hi = make_int2(max3i(o.p0.x, o.p1.x, o.p2.x), max3i(o.p0.y, o.p1.y, o.p2.y));
    return o;
}

__device__ __forceinline__ S64 cross2(S32 ax, S32 ay, S32 bx, S32 by) { return (S64)ax * by - (S64)ay * bx; }

// prepareTriangle (TriangleSetup.inl:38-100): 0 visible, 1 backfacing, 2 between samples.
// The area is formed in 64 bits (equal to the reference's S32 product up to
// 2048-px viewports, overflow-free beyond).
template <int S>
__device__ __forceinline__ int prepareTriangle(const SnapOut& t, S32 width, S32 height, int2& d1, int2& d2, S64& area) {
    d1 = make_int2((S32)((U32)t.p1.x - (U32)t.p0.x), (S32)((U32)t.p1.y - (U32)t.p0.y));
    d2 = make_int2((S32)((U32)t.p2.x - (U32)t.p0.x), (S32)((U32)t.p2.y - (U32)t.p0.y));
    area = (S64)d1.x * d2.y - (S64)d1.y * d2.x;
    if (area <= 0) return 1;
    const S32 sampleSize = 1 << (kSubpixelLog2 - S);
    S32 biasX = (width << (kSubpixelLog2 - 1)) - (sampleSize >> 1);
    S32 biasY = (height << (kSubpixelLog2 - 1)) - (sampleSize >> 1);
    S32 lox = (S32)((U32)t.lo.x + (U32)(sampleSize - 1) + (U32)biasX) & -sampleSize;
    S32 loy = (S32)((U32)t.lo.y + (U32)(sampleSize - 1) + (U32)biasY) & -sampleSize;
    S32 hix = (S32)((U32)t.hi.x + (U32)biasX) & -sampleSize;
    S32 hiy = (S32)((U32)t.hi.y + (U32)biasY) & -sampleSize;
    if (lox > hix || loy > hiy) return 2;
    S32 diff = (S32)((U32)hix + (U32)hiy - (U32)lox - (U32)loy);
    if (diff <= sampleSize) {
        S32 ax = t.p0.x + biasX - lox, ay = t.p0.y + biasY - loy;
        S32 bx = t.p1.x + biasX - lox, by = t.p1.y + biasY - loy;
        S32 cx = t.p2.x + biasX - lox, cy = t.p2.y + biasY - loy;
        if (cross2(ax, ay, bx, by) < 0 || cross2(bx, by, cx, cy) < 0 || cross2(cx, cy, ax, ay) < 0) {
            if (diff == 0) return 2;
            ax = t.p0.x + biasX - hix; ay = t.p0.y + biasY - hiy;
            bx = t.p1.x + biasX - hix; by = t.p1.y + biasY - hiy;
            cx = t.p2.x + biasX - hix; cy = t.p2.y + biasY - hiy;
            if (cross2(ax, ay, bx, by) < 0 || cross2(bx, by, cx, cy) < 0 || cross2(cx, cy, ax, ay) < 0) return 2;
        }
    }
    return 0;
}

// setupTriangle (TriangleSetup.inl:104-215): writes one header + data slot.
template <int S, U32 F>
__device__ __forceinline__ void setupTriangle(uint4* th, uint4* td, int3 vidx, float4 v0, float4 v1, float4 v2,
                                              float2 b0, float2 b1, float2 b2, const SnapOut& t,
                                              int2 d1, int2 d2, S64 area, S32 width, S32 height) {
    F32 areaRcp = 0.0f;
    int2 wv0 = make_int2(0, 0);
    if (F & (kRenderDepth | kRenderLerp)) {
        areaRcp = frcp(__ll2float_rn(area));
        wv0.x = t.p0.x + (width << (kSubpixelLog2 - 1));
        wv0.y = t.p0.y + (height << (kSubpixelLog2 - 1));
    }
    U32 zx = 0, zy = 0, zb = 0, zmin = 0, zslope = 0;
    if (F & kRenderDepth) {
        const F32 zcoef = (F32)(kDepthMax - kDepthMin) * 0.5f;
        const F32 zbias = (F32)(kDepthMax + kDepthMin) * 0.5f;
        F32 z0 = fadd(fmul(fmul(v0.z, zcoef), t.rcpW0), zbias);
        F32 z1 = fadd(fmul(fmul(v1.z, zcoef), t.rcpW1), zbias);
        F32 z2 = fadd(fmul(fmul(v2.z, zcoef), t.rcpW2), zbias);
        int2 zv0 = make_int2(wv0.x - (1 << (kSubpixelLog2 - S - 1)), wv0.y - (1 << (kSubpixelLog2 - S - 1)));
        setupPleq(z0, z1, z2, zv0, d1, d2, areaRcp, S, zx, zy, zb);
        zmin = f32_to_u32_sat(fsub(fminf(fminf(z0, z1), z2), (F32)lerpError(S)));
        if (S != 0) {
            U32 tmp = absWrap((S32)zx) + absWrap(max((S32)zy, -0x7FFFFFFF));
            const int sh = (S - 1 > 0) ? S - 1 : 0;
            zslope = tmp << sh;
            if ((zslope >> sh) != tmp) zslope = 0xFFFFFFFFu;
        }
    }
    U32 wx = 0, wy = 0, wb = 0, ux = 0, uy = 0, ub = 0, vx = 0, vy = 0, vb = 0;
    if (F & kRenderLerp) {
        F32 wcoef = fmul(fminf(fminf(v0.w, v1.w), v2.w), (F32)kBaryMax);
        F32 w0 = fmul(wcoef, t.rcpW0), w1 = fmul(wcoef, t.rcpW1), w2 = fmul(wcoef, t.rcpW2);
        setupPleq(w0, w1, w2, wv0, d1, d2, areaRcp, S + 1, wx, wy, wb);
        setupPleq(fmul(b0.x, w0), fmul(b1.x, w1), fmul(b2.x, w2), wv0, d1, d2, areaRcp, S + 1, ux, uy, ub);
        setupPleq(fmul(b0.y, w0), fmul(b1.y, w1), fmul(b2.y, w2), wv0, d1, d2, areaRcp, S + 1, vx, vy, vb);
    }
    td[0] = make_uint4(zx, zy, zb, zslope);
    td[1] = make_uint4(wx, wy, wb, ux);
    td[2] = make_uint4(uy, ub, vx, vy);
    td[3] = make_uint4(vb, (U32)vidx.x, (U32)vidx.y, (U32)vidx.z);
    U32 f01 = selectFlips(d1.x, d1.y);
    U32 f12 = selectFlips(d2.x - d1.x, d2.y - d1.y);
    U32 f20 = selectFlips(-d2.x, -d2.y);
    *th = make_uint4(((U32)t.p0.x & 0xFFFFu) | ((U32)t.p0.y << 16),
                     ((U32)t.p1.x & 0xFFFFu) | ((U32)t.p1.y << 16),
                     ((U32)t.p2.x & 0xFFFFu) | ((U32)t.p2.y << 16),
                     (zmin & 0xFFFFF000u) | (f01 << 6) | (f12 << 2) | (f20 >> 2));
}

__device__ __forceinline__ float4 lerpClip(float4 o, float4 a, float4 b, F32 bu, F32 bv) {
    return make_float4(fadd(fadd(o.x, fmul(a.x, bu)), fmul(b.x, bv)), fadd(fadd(o.y, fmul(a.y, bu)), fmul(b.y, bv)),
                       fadd(fadd(o.z, fmul(a.z, bu)), fmul(b.z, bv)), fadd(fadd(o.w, fmul(a.w, bu)), fmul(b.w, bv)));
}

// Clip path of triangleSetupImpl (TriangleSetup.inl:326-412), out of line so
// the common path keeps its registers.
template <int S, U32 F>
__device__ __noinline__ void setupClipped(const DrawDev& d, S64 gt, int3 vidx, float4 v0, float4 v1, float4 v2,
                                          S32 width, S32 height) {
    int2 d1, d2;
    S64 area;
    float4 ov0 = v0;
    float4 od1 = make_float4(fsub(v1.x, v0.x), fsub(v1.y, v0.y), fsub(v1.z, v0.z), fsub(v1.w, v0.w));
    float4 od2 = make_float4(fsub(v2.x, v0.x), fsub(v2.y, v0.y), fsub(v2.z, v0.z), fsub(v2.w, v0.w));
    F32 bary[18];
    int numVerts = clipTriangle(bary, &ov0.x, &v1.x, &v2.x, &od1.x, &od2.x);
    float4 c0 = lerpClip(ov0, od1, od2, bary[0], bary[1]);
    float4 c1 = lerpClip(ov0, od1, od2, bary[2], bary[3]);
    float4 tc1 = c1;

    int numSubtris = 0;
    for (int i = 2; i < numVerts; i++) {
        float4 c2 = lerpClip(ov0, od1, od2, bary[i * 2], bary[i * 2 + 1]);
        SnapOut sn = snapTriangle(c0, c1, c2, width, height);
        if (prepareTriangle<S>(sn, width, height, d1, d2, area) == 0) numSubtris++;
        c1 = c2;
    }
    d.triSubtris[gt] = (uint8_t)numSubtris;

    S64 base = gt;
    if (numSubtris > 1) {
        base = d.totalTris + atomicAdd(&d.counters->extraSubtris, numSubtris);
        d.triHeader[gt].w = (U32)base;
        if (base + numSubtris > d.maxSubtris) {
            atomicOr(&d.counters->overflow, kOverflowSubtris);
            numVerts = 0;
        }
    }
    c1 = tc1;
    for (int i = 2; i < numVerts; i++) {
        float4 c2 = lerpClip(ov0, od1, od2, bary[i * 2], bary[i * 2 + 1]);
        SnapOut sn = snapTriangle(c0, c1, c2, width, height);
        if (prepareTriangle<S>(sn, width, height, d1, d2, area) == 0) {
            setupTriangle<S, F>(&d.triHeader[base], &d.triData[base * 4], vidx, c0, c1, c2,
                                make_float2(bary[0], bary[1]), make_float2(bary[i * 2 - 2], bary[i * 2 - 1]),
                                make_float2(bary[i * 2], bary[i * 2 + 1]), sn, d1, d2, area, width, height);
            base++;
        }
        c1 = c2;
    }
}

// Clip position of vertex i: its record's clipPos, or, with the fused vertex
// transform, mvp * (model[i], 1) with each row summed left to right from zero
// as vertexShader_passthrough (PassThrough.cu:16-35, Math.hpp:990-1001)
// writes it, so both give the same bits. d.mvp lives in the kernel's
// parameter space.
__device__ __forceinline__ float4 transformModel(const DrawDev& d, int i) {
    const float* p = d.model + (S64)i * d.modelStride;
    F32 x, y, z;
    if (d.modelVec4) {
        const float4 q = __ldg((const float4*)p);
        x = q.x, y = q.y, z = q.z;
    } else {
        x = __ldg(p + 0), y = __ldg(p + 1), z = __ldg(p + 2);
    }
    F32 r[4];
#pragma unroll
    for (int row = 0; row < 4; row++)
        r[row] = fadd(fadd(fadd(fadd(0.0f, fmul(d.mvp[row * 4 + 0], x)), fmul(d.mvp[row * 4 + 1], y)),
                           fmul(d.mvp[row * 4 + 2], z)),
                      fmul(d.mvp[row * 4 + 3], 1.0f));
    return make_float4(r[0], r[1], r[2], r[3]);
}

__device__ __forceinline__ void fetchClip(const DrawDev& d, const float4* verts, S32 stride4, int3 vidx, float4& v0,
                                          float4& v1, float4& v2) {
    if (d.model == nullptr) {
        v0 = __ldg(&verts[(S64)vidx.x * stride4]);
        v1 = __ldg(&verts[(S64)vidx.y * stride4]);
        v2 = __ldg(&verts[(S64)vidx.z * stride4]);
    } else {
        v0 = transformModel(d, vidx.x);
        v1 = transformModel(d, vidx.y);
        v2 = transformModel(d, vidx.z);
    }
}

// Resident setup CTAs per SM the compiler must allow (register budget):
// five (48 registers). Six (40 registers, 52 bytes
// spilled) measured slower on the soup and the 4x MSAA grid (setup 36.7 ->
// 38.4 us and 0.168 -> 0.172 ms) and level on the fly-through.
#ifndef CR_SETUP_MIN_BLOCKS
#define CR_SETUP_MIN_BLOCKS 5
#endif

// triangleSetupImpl (TriangleSetup.inl:219-417), over the triangle range of
// one pipe group [triBegin, triEnd) (global triangle slots).
template <int S, U32 F>
__global__ void __launch_bounds__(256, CR_SETUP_MIN_BLOCKS) setupKernel(DrawDev d, int instBegin, int instEnd, S64 triBegin, S64 triEnd) {
    pdlWait();
    pdlTrigger();
    S64 gt = triBegin + (S64)blockIdx.x * 256 + threadIdx.x;
    if (gt >= triEnd) return;
    int ii = instBegin + findInstance64(d.triPrefix + instBegin, instEnd - instBegin, gt);
    const InstanceDev* in = &d.inst[ii];
    const S32 width = __ldg(&in->width), height = __ldg(&in->height), stride4 = __ldg(&in->stride4);
    const int* indices = (const int*)__ldg((const unsigned long long*)&in->indices);
    const float4* verts = (const float4*)__ldg((const unsigned long long*)&in->vertices);
    S64 t = gt - __ldg(&in->triBase);

    int3 vidx = make_int3(__ldg(&indices[3 * t + 0]), __ldg(&indices[3 * t + 1]), __ldg(&indices[3 * t + 2]));
    float4 v0, v1, v2;
    fetchClip(d, verts, stride4, vidx, v0, v1, v2);

    // Outside view frustum => cull (TriangleSetup.inl:262-281).
    if ((v0.w < fabsf(v0.x)) | (v0.w < fabsf(v0.y)) | (v0.w < fabsf(v0.z))) {
        if (((v0.w < +v0.x) & (v1.w < +v1.x) & (v2.w < +v2.x)) |
            ((v0.w < -v0.x) & (v1.w < -v1.x) & (v2.w < -v2.x)) |
            ((v0.w < +v0.y) & (v1.w < +v1.y) & (v2.w < +v2.y)) |
            ((v0.w < -v0.y) & (v1.w < -v1.y) & (v2.w < -v2.y)) |
            ((v0.w < +v0.z) & (v1.w < +v1.z) & (v2.w < +v2.z)) |
            ((v0.w < -v0.z) & (v1.w < -v1.z) & (v2.w < -v2.z))) {
            d.triSubtris[gt] = 0;
            return;
        }
    }

    int2 d1, d2;
    S64 area;
    // Inside depth range and small enough => fast path (TriangleSetup.inl:285-322).
    if ((v0.w >= fabsf(v0.z)) & (v1.w >= fabsf(v1.z)) & (v2.w >= fabsf(v2.z))) {
        SnapOut sn = snapTriangle(v0, v1, v2, width, height);
        S32 loxy = min(sn.lo.x, sn.lo.y);
        S32 hixy = max(sn.hi.x, sn.hi.y);
        const S32 aabbLimit = (1 << (kMaxViewportLog2Ref + kSubpixelLog2)) - 1;
        if (loxy >= -32768 && hixy <= 32767 && hixy - loxy <= aabbLimit) {
            int res = prepareTriangle<S>(sn, width, height, d1, d2, area);
            d.triSubtris[gt] = (res == 0) ? 1 : 0;
            if (res == 0)
                setupTriangle<S, F>(&d.triHeader[gt], &d.triData[gt * 4], vidx, v0, v1, v2,
                                    make_float2(0.0f, 0.0f), make_float2(1.0f, 0.0f), make_float2(0.0f, 1.0f),
                                    sn, d1, d2, area, width, height);
            return;
        }
    }

    // Clip to the view frustum (TriangleSetup.inl:326-412); rare, kept out of line.
    setupClipped<S, F>(d, gt, vidx, v0, v1, v2, width, height);
}

}  // namespace cr
