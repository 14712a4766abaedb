// vertex.cu -- the vertex stage before the rasterizer: clip = MVP * (model, 1)
// per vertex, the reference's vertexShader_passthrough (test/shader/
// PassThrough.cu:16-35) with Mat4f * Vec4f evaluated as the reference's
// framework writes it (Math.hpp:990-1001: r[i] = sum over j of m(i, j) * v[j],
// accumulated left to right from zero, each operation rounded on its own).
// Per-vertex RGBA colours (optional) are copied behind the position to form
// GouraudVertex records.
#include "cudaraster.h"
#include "cudaraster/ShaderMath.hpp"
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
// products and matrix rows summed left to right from zero), one rounded
// operation at a time; normalize and powf are the exactly specified crNormalize
// and crPow of ShaderMath.hpp, so the CPU oracle matches every bit.
namespace cr {

struct VertexConstants {
    float posToClip[16];       // row-major
    float posToCamera[16];
    float normalToCamera[9];
};

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

// InputVertex records (Shaders.hpp: modelPos, modelNormal, texCoord; 8
// floats) -> GouraudVertex records (clipPos, lit colour). Materials start with
// the reference's Material fields diffuseColor (rgba), specularColor (rgb) and
// glossiness; records are materialStride floats apart.
__global__ void __launch_bounds__(256) vertexGouraudKernel(const float* __restrict__ in, int64_t n, VertexConstants c,
                                                           const float* __restrict__ materials, int materialStride,
                                                           int numMaterials, const int* __restrict__ materialIdx,
                                                           float4* __restrict__ out) {
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
    const float* mat = materials + (int64_t)mi * materialStride;
    const FW::Vec3f color = FW::evaluateLighting(
        FW::Vec3f(cameraPos[0], cameraPos[1], cameraPos[2]), FW::Vec3f(cameraNormal[0], cameraNormal[1], cameraNormal[2]),
        FW::Vec3f(__ldg(mat + 4), __ldg(mat + 5), __ldg(mat + 6)), __ldg(mat + 7),
        FW::Vec3f(__ldg(mat + 0), __ldg(mat + 1), __ldg(mat + 2)));
    out[i * 2 + 0] = make_float4(clip[0], clip[1], clip[2], clip[3]);
    out[i * 2 + 1] = make_float4(color.x, color.y, color.z, __ldg(mat + 3));
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

// The exact power over arrays (for its tests): out[i] = x[i]^y[i].
__global__ void powExactKernel(const float* __restrict__ x, const float* __restrict__ y, float* __restrict__ out,
                               int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = FW::crPow(x[i], y[i]);
}

static VertexConstants toConstants(const cr_vertex_constants* k) {
    VertexConstants c;
    for (int j = 0; j < 16; j++) c.posToClip[j] = k->pos_to_clip[j];
    for (int j = 0; j < 16; j++) c.posToCamera[j] = k->pos_to_camera[j];
    for (int j = 0; j < 9; j++) c.normalToCamera[j] = k->normal_to_camera[j];
    return c;
}

static bool gridFits(int64_t n) { return (n + 255) / 256 <= 0x7FFFFFFF; }

}  // namespace cr

extern "C" cr_status cr_vertex_shader_gouraud(const void* in_vertices, int64_t num_vertices,
                                              const cr_vertex_constants* constants, const void* materials,
                                              int32_t material_stride_bytes, int32_t num_materials,
                                              const int32_t* vertex_material_idx, void* out_vertices, void* stream) {
    if (material_stride_bytes == 0) material_stride_bytes = 32;
    if (!in_vertices || !constants || !materials || num_materials < 1 || !vertex_material_idx || !out_vertices ||
        num_vertices < 0 || !cr::gridFits(num_vertices) || material_stride_bytes < 32 || (material_stride_bytes & 3) ||
        ((uintptr_t)out_vertices & 15) || ((uintptr_t)in_vertices & 3) || ((uintptr_t)materials & 3))
        return CR_ERR_INVALID_ARGUMENT;
    if (num_vertices == 0) return CR_OK;
    const int64_t grid = (num_vertices + 255) / 256;
    cr::vertexGouraudKernel<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(
        (const float*)in_vertices, num_vertices, cr::toConstants(constants), (const float*)materials,
        material_stride_bytes / 4, num_materials, vertex_material_idx, (float4*)out_vertices);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

extern "C" cr_status cr_vertex_shader_tex_phong(const void* in_vertices, int64_t num_vertices,
                                               const cr_vertex_constants* constants, void* out_vertices,
                                               void* stream) {
    if (!in_vertices || !constants || !out_vertices || num_vertices < 0 || !cr::gridFits(num_vertices) ||
        ((uintptr_t)out_vertices & 15) || ((uintptr_t)in_vertices & 3))
        return CR_ERR_INVALID_ARGUMENT;
    if (num_vertices == 0) return CR_OK;
    const int64_t grid = (num_vertices + 255) / 256;
    cr::vertexTexPhongKernel<<<(unsigned)grid, 256, 0, (cudaStream_t)stream>>>(
        (const float*)in_vertices, num_vertices, cr::toConstants(constants), (float4*)out_vertices);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

extern "C" cr_status cr_pow_exact(const float* x, const float* y, float* out, int64_t n, void* stream) {
    if (!x || !y || !out || n < 0 || !cr::gridFits(n)) return CR_ERR_INVALID_ARGUMENT;
    if (n == 0) return CR_OK;
    cr::powExactKernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, y, out, n);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}
