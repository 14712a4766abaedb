// vertex.cu -- the vertex stage before the rasterizer: clip = MVP * (model, 1)
// per vertex, the reference's vertexShader_passthrough (test/shader/
// PassThrough.cu:16-35) with Mat4f * Vec4f evaluated as the reference's
// framework writes it (Math.hpp:990-1001: r[i] = sum over j of m(i, j) * v[j],
// accumulated left to right from zero, each operation rounded on its own).
// Per-vertex RGBA colours (optional) are copied behind the position to form
// GouraudVertex records.
#include "cudaraster.h"
#include "cudaraster/detail/device.cuh"

namespace cr {

struct Mvp {
    float m[16];  // row-major
};

__global__ void __launch_bounds__(256) vertexPassthroughKernel(const float* __restrict__ model, int modelStride,
                                                               const float* __restrict__ colors, int colorStride,
                                                               float4* __restrict__ out, int outStride4, int64_t n,
                                                               Mvp mvp) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = model + i * modelStride;
    const float v[4] = {__ldg(p + 0), __ldg(p + 1), __ldg(p + 2), 1.0f};
    float r[4];
#pragma unroll
    for (int row = 0; row < 4; row++) {
        float acc = 0.0f;
#pragma unroll
        for (int c = 0; c < 4; c++) acc = fadd(acc, fmul(mvp.m[row * 4 + c], v[c]));
        r[row] = acc;
    }
    float4* o = out + i * outStride4;
    o[0] = make_float4(r[0], r[1], r[2], r[3]);
    if (colors && outStride4 > 1) {
        const float* c = colors + i * colorStride;
        o[1] = make_float4(__ldg(c + 0), __ldg(c + 1), __ldg(c + 2), __ldg(c + 3));
    }
}

}  // namespace cr

extern "C" cr_status cr_vertex_shader_passthrough(const float* model, int32_t model_stride, const float* colors,
                                                  int32_t color_stride, void* out_vertices, int32_t out_stride_bytes,
                                                  int64_t num_vertices, const float* mvp_row_major, void* stream) {
    if (!model || !out_vertices || !mvp_row_major || num_vertices < 0 || model_stride < 3 ||
        (out_stride_bytes != 16 && out_stride_bytes != 32) || (colors && color_stride < 4) ||
        ((uintptr_t)out_vertices & 15))
        return CR_ERR_INVALID_ARGUMENT;
    if (num_vertices == 0) return CR_OK;
    cr::Mvp m;
    for (int k = 0; k < 16; k++) m.m[k] = mvp_row_major[k];
    int64_t grid = (num_vertices + 255) / 256;
    cr::vertexPassthroughKernel<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(
        model, model_stride, colors, color_stride, (float4*)out_vertices, out_stride_bytes / 16, num_vertices, m);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// vertexShader_gouraud and vertexShader_texPhong (test/shader/Shaders.cu:55-108)
// with evaluateLighting (Shaders.cu:37-50). The vector and matrix arithmetic
// follows the reference framework's C (Math.hpp:112-202, 990-1001: dot
// products and matrix rows summed left to right from zero, normalized(v) =
// v * (1 * rcp(length)), rcp(0) = 0), one rounded operation at a time. The
// reference compiles Shaders.cu with -use_fast_math, whose approximations
// cannot be reproduced, so sqrt is IEEE and powf is replaced by powExact: a
// power built from exact operations -- log2 by the atanh series
// log2(m) = (2 / ln 2) * sum t^(2k+1) / (2k+1), t = (m - 1) / (m + 1), for the
// mantissa m in [sqrt(1/2), sqrt(2)], and exp2 by the Taylor series of
// e^(f ln 2) around f = 1/2 -- within about 1e-5 relative of pow, and
// restated operation for operation by the oracle.
namespace cr {

struct VertexConstants {
    float posToClip[16];       // row-major
    float posToCamera[16];
    float normalToCamera[9];
};

__host__ __device__ constexpr U32 f32Bits(int e) { return (U32)(e + 127) << 23; }   // 2^e, e in [-126, 127]

__device__ __forceinline__ F32 log2Exact(F32 x) {   // x > 0, finite
    U32 b = __float_as_uint(x);
    S32 k = 0;
    if ((b >> 23) == 0u) {   // subnormal: scale by 2^24 first
        x = fmul(x, 16777216.0f);
        b = __float_as_uint(x);
        k = -24;
    }
    k += (S32)(b >> 23) - 127;
    F32 m = __uint_as_float((b & 0x7FFFFFu) | 0x3F800000u);   // [1, 2)
    if (m > 1.41421354f) {
        m = fmul(m, 0.5f);
        k += 1;
    }
    const F32 t = fdiv(fsub(m, 1.0f), fadd(m, 1.0f));
    const F32 t2 = fmul(t, t);
    F32 p = 0.26230818f;
    p = fadd(fmul(p, t2), 0.3205989f);
    p = fadd(fmul(p, t2), 0.41219857f);
    p = fadd(fmul(p, t2), 0.57707804f);
    p = fadd(fmul(p, t2), 0.9617967f);
    p = fadd(fmul(p, t2), 2.88539f);
    return fadd((F32)k, fmul(t, p));
}

__device__ __forceinline__ F32 exp2Exact(F32 z) {
    if (z != z) return z;
    if (z >= 128.0f) return __uint_as_float(0x7F800000u);
    if (!(z > -150.0f)) return 0.0f;
    const F32 n = floorf(z);
    const F32 f = fsub(fsub(z, n), 0.5f);   // [-0.5, 0.5)
    F32 p = 1.0178086e-07f;
    p = fadd(fmul(p, f), 1.3215487e-06f);
    p = fadd(fmul(p, f), 1.5252734e-05f);
    p = fadd(fmul(p, f), 1.540353e-04f);
    p = fadd(fmul(p, f), 1.3333558e-03f);
    p = fadd(fmul(p, f), 9.618129e-03f);
    p = fadd(fmul(p, f), 5.550411e-02f);
    p = fadd(fmul(p, f), 2.402265e-01f);
    p = fadd(fmul(p, f), 6.931472e-01f);
    p = fadd(fmul(p, f), 1.0f);
    p = fmul(p, 1.4142135f);
    S32 ni = (S32)n;
    if (ni < -126) {
        p = fmul(p, __uint_as_float(f32Bits(-64)));
        ni += 64;
    }
    return fmul(p, __uint_as_float(f32Bits(ni)));
}

// x^y for x >= 0 (the lighting's powf(max(-dot(I, R), 0), glossiness)).
__device__ __forceinline__ F32 powExact(F32 x, F32 y) {
    if (y == 0.0f) return 1.0f;
    if (!(x > 0.0f)) return y > 0.0f ? 0.0f : __uint_as_float(0x7F800000u);
    if (x == __uint_as_float(0x7F800000u)) return y > 0.0f ? x : 0.0f;
    return exp2Exact(fmul(y, log2Exact(x)));
}

template <int R, int C>
__device__ __forceinline__ void matVec(const float* m, const F32* v, F32* r) {
#pragma unroll
    for (int i = 0; i < R; i++) {
        F32 acc = 0.0f;
#pragma unroll
        for (int j = 0; j < C; j++) acc = fadd(acc, fmul(m[i * C + j], v[j]));
        r[i] = acc;
    }
}

__device__ __forceinline__ F32 dot3(const F32* a, const F32* b) {
    return fadd(fadd(fadd(0.0f, fmul(a[0], b[0])), fmul(a[1], b[1])), fmul(a[2], b[2]));
}

__device__ __forceinline__ void normalize3(const F32* v, F32* r) {
    const F32 len = __fsqrt_rn(dot3(v, v));
    const F32 s = fmul(1.0f, len != 0.0f ? fdiv(1.0f, len) : 0.0f);
#pragma unroll
    for (int k = 0; k < 3; k++) r[k] = fmul(v[k], s);
}

// InputVertex records (Shaders.hpp: modelPos, modelNormal, texCoord; 8
// floats) -> GouraudVertex records (clipPos, lit colour).
__global__ void __launch_bounds__(256) vertexGouraudKernel(const float* __restrict__ in, int64_t n, VertexConstants c,
                                                           const float* __restrict__ materials, int numMaterials,
                                                           const int* __restrict__ materialIdx, float4* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = in + i * 8;
    const F32 pos[4] = {__ldg(v + 0), __ldg(v + 1), __ldg(v + 2), 1.0f};
    const F32 nrm[3] = {__ldg(v + 3), __ldg(v + 4), __ldg(v + 5)};
    F32 cameraPos[3], cameraNormal[3], clip[4];
    matVec<3, 4>(c.posToCamera, pos, cameraPos);
    matVec<3, 3>(c.normalToCamera, nrm, cameraNormal);
    matVec<4, 4>(c.posToClip, pos, clip);
    const int mi = min(max(__ldg(materialIdx + i), 0), numMaterials - 1);
    const float* mat = materials + (int64_t)mi * 8;   // diffuse rgba, specular rgb, glossiness
    // evaluateLighting (Shaders.cu:37-50).
    F32 I[3], N[3], R[3];
    normalize3(cameraPos, I);
    normalize3(cameraNormal, N);
    const F32 dotIN = dot3(I, N);
    const F32 twice = fmul(dotIN, 2.0f);
#pragma unroll
    for (int k = 0; k < 3; k++) R[k] = fsub(I[k], fmul(N[k], twice));
    const F32 diffuseCoef = fadd(fmul(fmaxf(-dotIN, 0.0f), 0.75f), 0.25f);
    const F32 specularCoef = powExact(fmaxf(-dot3(I, R), 0.0f), __ldg(mat + 7));
    F32 color[3];
#pragma unroll
    for (int k = 0; k < 3; k++) color[k] = fadd(fmul(__ldg(mat + k), diffuseCoef), fmul(__ldg(mat + 4 + k), specularCoef));
    out[i * 2 + 0] = make_float4(clip[0], clip[1], clip[2], clip[3]);
    out[i * 2 + 1] = make_float4(color[0], color[1], color[2], __ldg(mat + 3));
}

// InputVertex records -> ShadedVertex_texPhong records (clipPos, cameraPos,
// cameraNormal (w 0), texCoord (z 0, w 1)).
__global__ void __launch_bounds__(256) vertexTexPhongKernel(const float* __restrict__ in, int64_t n, VertexConstants c,
                                                            float4* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = in + i * 8;
    const F32 pos[4] = {__ldg(v + 0), __ldg(v + 1), __ldg(v + 2), 1.0f};
    const F32 nrm[3] = {__ldg(v + 3), __ldg(v + 4), __ldg(v + 5)};
    F32 clip[4], cameraPos[4], cameraNormal[3];
    matVec<4, 4>(c.posToClip, pos, clip);
    matVec<4, 4>(c.posToCamera, pos, cameraPos);
    matVec<3, 3>(c.normalToCamera, nrm, cameraNormal);
    out[i * 4 + 0] = make_float4(clip[0], clip[1], clip[2], clip[3]);
    out[i * 4 + 1] = make_float4(cameraPos[0], cameraPos[1], cameraPos[2], cameraPos[3]);
    out[i * 4 + 2] = make_float4(cameraNormal[0], cameraNormal[1], cameraNormal[2], 0.0f);
    out[i * 4 + 3] = make_float4(__ldg(v + 6), __ldg(v + 7), 0.0f, 1.0f);
}

// Exact power over arrays (for its tests): out[i] = x[i]^y[i].
__global__ void powExactKernel(const float* __restrict__ x, const float* __restrict__ y, float* __restrict__ out,
                               int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = powExact(x[i], y[i]);
}

static VertexConstants toConstants(const cr_vertex_constants* k) {
    VertexConstants c;
    for (int j = 0; j < 16; j++) c.posToClip[j] = k->pos_to_clip[j];
    for (int j = 0; j < 16; j++) c.posToCamera[j] = k->pos_to_camera[j];
    for (int j = 0; j < 9; j++) c.normalToCamera[j] = k->normal_to_camera[j];
    return c;
}

}  // namespace cr

extern "C" cr_status cr_vertex_shader_gouraud(const void* in_vertices, int64_t num_vertices,
                                              const cr_vertex_constants* constants, const void* materials,
                                              int32_t num_materials, const int32_t* vertex_material_idx,
                                              void* out_vertices, void* stream) {
    if (!in_vertices || !constants || !materials || num_materials < 1 || !vertex_material_idx || !out_vertices ||
        num_vertices < 0 || ((uintptr_t)out_vertices & 15) || ((uintptr_t)in_vertices & 3) || ((uintptr_t)materials & 3))
        return CR_ERR_INVALID_ARGUMENT;
    if (num_vertices == 0) return CR_OK;
    const int64_t grid = (num_vertices + 255) / 256;
    cr::vertexGouraudKernel<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(
        (const float*)in_vertices, num_vertices, cr::toConstants(constants), (const float*)materials, num_materials,
        vertex_material_idx, (float4*)out_vertices);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

extern "C" cr_status cr_vertex_shader_tex_phong(const void* in_vertices, int64_t num_vertices,
                                               const cr_vertex_constants* constants, void* out_vertices,
                                               void* stream) {
    if (!in_vertices || !constants || !out_vertices || num_vertices < 0 || ((uintptr_t)out_vertices & 15) ||
        ((uintptr_t)in_vertices & 3))
        return CR_ERR_INVALID_ARGUMENT;
    if (num_vertices == 0) return CR_OK;
    const int64_t grid = (num_vertices + 255) / 256;
    cr::vertexTexPhongKernel<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(
        (const float*)in_vertices, num_vertices, cr::toConstants(constants), (float4*)out_vertices);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

extern "C" cr_status cr_pow_exact(const float* x, const float* y, float* out, int64_t n, void* stream) {
    if (!x || !y || !out || n < 0) return CR_ERR_INVALID_ARGUMENT;
    if (n == 0) return CR_OK;
    cr::powExactKernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, y, out, n);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}
