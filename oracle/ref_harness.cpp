/*
 * ref_harness.cpp -- compiles the reference rasterizer's own device code
 * (tcoppex/cudaraster-linux, src/cudaraster/cuda/PixelPipe.inl and the
 * stage .inl files it includes) for the host, in place, and exposes a few of
 * its functions through a C interface.
 *
 * TEST INFRASTRUCTURE ONLY. Built by oracle/Makefile (target `ref`) into
 * oracle/_ref/ when the reference sources are present; its outputs become the
 * golden vectors in tests/golden/ (tests/golden/make_golden.py).
 *
 * The reference's device code is plain C++ apart from inline-PTX helpers
 * (Util.hpp:72-151), CUDA intrinsics and legacy texture/surface references.
 * Those are supplied below as host functions that follow the PTX ISA
 * semantics of the instruction each helper wraps (cvt saturation and
 * rounding, video-instruction byte/half selection, carry chains, prmt byte
 * selection, fma rounding modes). Everything else -- snapping, culling,
 * clipping, plane equations, coverage masks, barycentrics, shading, blending
 * -- is the reference's own source. Only per-thread functions are called;
 * the warp-synchronous loops of the bin/coarse/fine stages are compiled but
 * never run.
 */
#include "ref_shim.h"

#include "cudaraster/cuda/PixelPipe.inl"

// Module globals declared by PixelPipe.inl:27-37.
namespace FW {
extern "C" {
CRParams c_crParams;
CRAtomics g_crAtomics;
S32 c_profLaunchIdx;
CUdeviceptr c_profData;
texture<float4, 1> t_vertexBuffer;
texture<uint4, 1> t_triHeader;
texture<uint4, 1> t_triData;
surface<void, 2> s_colorBuffer;
surface<void, 2> s_depthBuffer;
}
}  // namespace FW

using namespace FW;

namespace {
template <class V, int S, U32 F>
void run_setup_impl(int numTris) {
    blockDim = dim3(32, CR_SETUP_WARPS, 1);
    int perBlock = 32 * CR_SETUP_WARPS;
    gridDim = dim3((numTris + perBlock - 1) / perBlock, 1, 1);
    for (unsigned b = 0; b < gridDim.x; b++)
        for (unsigned y = 0; y < CR_SETUP_WARPS; y++)
            for (unsigned x = 0; x < 32; x++) {
                blockIdx = make_uint3(b, 0, 0);
                threadIdx = make_uint3(x, y, 0);
                triangleSetupImpl<V, S, F>();
            }
}

template <class V, int S>
void run_setup_flags(unsigned flags, int numTris) {
    switch (flags & 3) {
    case 0: run_setup_impl<V, S, 0>(numTris); break;
    case 1: run_setup_impl<V, S, 1>(numTris); break;
    case 2: run_setup_impl<V, S, 2>(numTris); break;
    default: run_setup_impl<V, S, 3>(numTris); break;
    }
}

template <class V>
void run_setup_samples(int s, unsigned flags, int numTris) {
    switch (s) {
    case 0: run_setup_flags<V, 0>(flags, numTris); break;
    case 1: run_setup_flags<V, 1>(flags, numTris); break;
    case 2: run_setup_flags<V, 2>(flags, numTris); break;
    default: run_setup_flags<V, 3>(flags, numTris); break;
    }
}

volatile U64 g_lut[CR_COVER8X8_LUT_SIZE];
bool g_lutReady = false;
void ensure_lut() {
    if (g_lutReady) return;
    blockDim = dim3(1, 1, 1);
    threadIdx = make_uint3(0, 0, 0);
    cover8x8_setupLUT(g_lut);
    g_lutReady = true;
}

template <int S, U32 F>
U32 run_gouraud(int triIdx, int dataIdx, int px, int py, U32 centroid) {
    static volatile U32 shared[32];
    threadIdx = make_uint3(0, 0, 0);
    GouraudShader fs;
    runFragmentShader<GouraudVertex, GouraudShader, S, F>(fs, triIdx, dataIdx, px, py, centroid, shared);
    return fs.m_color;
}
}  // namespace

extern "C" {

// Runs triangleSetupImpl (TriangleSetup.inl:219-417) over a whole draw.
// vertices: GouraudVertex (32 B) or ShadedVertexBase (16 B) records.
int ref_triangle_setup(int s, unsigned flags, int width, int height, int vertexStride,
                       const float* vertices, const int* indices, int numTris,
                       unsigned char* triSubtris, unsigned int* headers, unsigned int* data,
                       int maxSubtris) {
    std::memset(&c_crParams, 0, sizeof(c_crParams));
    c_crParams.numTris = numTris;
    c_crParams.indexBuffer = (CUdeviceptr)(uintptr_t)indices;
    c_crParams.viewportWidth = width;
    c_crParams.viewportHeight = height;
    c_crParams.maxSubtris = maxSubtris;
    c_crParams.triSubtris = (CUdeviceptr)(uintptr_t)triSubtris;
    c_crParams.triHeader = (CUdeviceptr)(uintptr_t)headers;
    c_crParams.triData = (CUdeviceptr)(uintptr_t)data;
    g_crAtomics.numSubtris = numTris;
    t_vertexBuffer.ptr = (const float4*)vertices;
    if (vertexStride == 16)
        run_setup_samples<ShadedVertexBase>(s, flags, numTris);
    else
        run_setup_samples<GouraudVertex>(s, flags, numTris);
    return g_crAtomics.numSubtris;
}

unsigned long long ref_cover8x8_exact_ref(int ox, int oy, int dx, int dy) { return cover8x8_exact_ref(ox, oy, dx, dy); }
unsigned long long ref_cover8x8_conservative_ref(int ox, int oy, int dx, int dy) { return cover8x8_conservative_ref(ox, oy, dx, dy); }
unsigned long long ref_cover8x8_exact_fast(int ox, int oy, int dx, int dy) {
    ensure_lut();
    return cover8x8_exact_fast(ox, oy, dx, dy, cover8x8_selectFlips(dx, dy), g_lut);
}
unsigned long long ref_cover8x8_conservative_fast(int ox, int oy, int dx, int dy) {
    ensure_lut();
    return cover8x8_conservative_fast(ox, oy, dx, dy, cover8x8_selectFlips(dx, dy), g_lut);
}
unsigned long long ref_cover8x8_exact_noLUT(int ox, int oy, int dx, int dy) { return cover8x8_exact_noLUT(ox, oy, dx, dy); }
unsigned int ref_coverMSAA_ref(int s, int ox, int oy, int dx, int dy) { return coverMSAA_ref(s, ox, oy, dx, dy); }
unsigned int ref_coverMSAA_fast(int s, int ox, int oy, int dx, int dy) { return coverMSAA_fast(s, ox, oy, dx, dy); }

// FineRaster.inl:244-280 / 284-305 on one header.
unsigned long long ref_triangle_pixel_coverage(int s, const unsigned int* header, int tileX, int tileY,
                                               int width, int height) {
    ensure_lut();
    c_crParams.viewportWidth = width;
    c_crParams.viewportHeight = height;
    uint4 h = make_uint4(header[0], header[1], header[2], header[3]);
    switch (s) {
    case 0: return trianglePixelCoverage<0>(h, tileX, tileY, g_lut);
    case 1: return trianglePixelCoverage<1>(h, tileX, tileY, g_lut);
    case 2: return trianglePixelCoverage<2>(h, tileX, tileY, g_lut);
    default: return trianglePixelCoverage<3>(h, tileX, tileY, g_lut);
    }
}
unsigned int ref_triangle_sample_coverage(int s, const unsigned int* header, int px, int py,
                                          int width, int height) {
    c_crParams.viewportWidth = width;
    c_crParams.viewportHeight = height;
    uint4 h = make_uint4(header[0], header[1], header[2], header[3]);
    switch (s) {
    case 1: return triangleSampleCoverage<1>(h, px, py);
    case 2: return triangleSampleCoverage<2>(h, px, py);
    default: return triangleSampleCoverage<3>(h, px, py);
    }
}

void ref_setup_pleq(const float* values, const int* v0, const int* d1, const int* d2,
                    float areaRcp, int s, unsigned int* out) {
    uint3 r = setupPleq(make_float3(values[0], values[1], values[2]), make_int2(v0[0], v0[1]),
                        make_int2(d1[0], d1[1]), make_int2(d2[0], d2[1]), areaRcp, s);
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

unsigned int ref_to_abgr(float r, float g, float b, float a) { return toABGR(make_float4(r, g, b, a)); }
unsigned int ref_host_to_abgr(float r, float g, float b, float a) { return Vec4f(r, g, b, a).toABGR(); }
unsigned int ref_encode_depth(unsigned int d) { return encodeDepth(d); }
unsigned int ref_decode_depth(unsigned int d) { return decodeDepth(d); }
unsigned int ref_select_flips(int dx, int dy) { return cover8x8_selectFlips(dx, dy); }
int ref_select_msaa_centroid(int s, unsigned int mask) { return selectMSAACentroid(s, mask); }
void ref_centroid_lut(int s, unsigned char* lut) {
    static volatile U8 tmp[256];
    blockDim = dim3(32, 1, 1);
    for (unsigned x = 0; x < 32; x++) {
        threadIdx = make_uint3(x, 0, 0);
        switch (s) {
        case 0: setupCentroidLUT<0>(tmp); break;
        case 1: setupCentroidLUT<1>(tmp); break;
        case 2: setupCentroidLUT<2>(tmp); break;
        default: setupCentroidLUT<3>(tmp); break;
        }
    }
    for (int i = 0; i < (1 << (1 << s)); i++) lut[i] = tmp[i];
}
int ref_clip_triangle(float* bary, const float* v0, const float* v1, const float* v2,
                      const float* d1, const float* d2) {
    return clipTriangleWithFrustum(bary, v0, v1, v2, d1, d2);
}

unsigned int ref_blend(int mode, unsigned int src, unsigned int dst, int* writeColor) {
    threadIdx = make_uint3(0, 0, 0);
    switch (mode) {
    case 0: { BlendReplace b; runBlendShader(b, 0, 0, 0, 0, src, dst); *writeColor = b.m_writeColor; return b.m_color; }
    case 1: { BlendSrcOver b; runBlendShader(b, 0, 0, 0, 0, src, dst); *writeColor = b.m_writeColor; return b.m_color; }
    case 2: { BlendAdditive b; runBlendShader(b, 0, 0, 0, 0, src, dst); *writeColor = b.m_writeColor; return b.m_color; }
    default: { BlendDepthOnly b; runBlendShader(b, 0, 0, 0, 0, src, dst); *writeColor = b.m_writeColor; return b.m_color; }
    }
}

void ref_compute_barys(int s, const int* w, const int* u, const int* v, int sx, int sy, float* out) {
    Vec3f b, bdx, bdy;
    Vec3i W(w[0], w[1], w[2]), U(u[0], u[1], u[2]), V(v[0], v[1], v[2]);
    switch (s) {
    case 0: computeBarys<0>(b, bdx, bdy, W, U, V, sx, sy); break;
    case 1: computeBarys<1>(b, bdx, bdy, W, U, V, sx, sy); break;
    case 2: computeBarys<2>(b, bdx, bdy, W, U, V, sx, sy); break;
    default: computeBarys<3>(b, bdx, bdy, W, U, V, sx, sy); break;
    }
    for (int i = 0; i < 3; i++) { out[i] = b[i]; out[3 + i] = bdx[i]; out[6 + i] = bdy[i]; }
}

int ref_find_bit(unsigned long long mask, int idx, int quads) {
    threadIdx = make_uint3(0, 0, 0);
    return quads ? findBit<RenderModeFlag_EnableQuads>(mask, idx) : findBit<0>(mask, idx);
}

// runFragmentShader (FineRaster.inl:48-119) + GouraudShader::run (PixelPipe.inl:65-69).
// triData: 16 words per slot; vertices: GouraudVertex records.
unsigned int ref_gouraud_fragment(int s, unsigned flags, const unsigned int* triData,
                                  const float* vertices, int triIdx, int dataIdx,
                                  int px, int py, unsigned int centroid) {
    t_triData.ptr = (const uint4*)triData;
    t_vertexBuffer.ptr = (const float4*)vertices;
    bool lerp = (flags & 2) != 0;
    switch (s * 2 + (lerp ? 1 : 0)) {
    case 0: return run_gouraud<0, 1>(triIdx, dataIdx, px, py, centroid);
    case 1: return run_gouraud<0, 3>(triIdx, dataIdx, px, py, centroid);
    case 2: return run_gouraud<1, 1>(triIdx, dataIdx, px, py, centroid);
    case 3: return run_gouraud<1, 3>(triIdx, dataIdx, px, py, centroid);
    case 4: return run_gouraud<2, 1>(triIdx, dataIdx, px, py, centroid);
    case 5: return run_gouraud<2, 3>(triIdx, dataIdx, px, py, centroid);
    case 6: return run_gouraud<3, 1>(triIdx, dataIdx, px, py, centroid);
    default: return run_gouraud<3, 3>(triIdx, dataIdx, px, py, centroid);
    }
}

void ref_perspective(float fov, float n, float f, float* out) {
    Mat4f m = Mat4f::perspective(fov, n, f);
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[r * 4 + c] = m.get(r, c);
}

}  // extern "C"
