// vertex.cu -- the vertex stage before the rasterizer: the reference's example
// vertex shaders. vertexShader_passthrough (test/shader/PassThrough.cu:16-35):
// clip = MVP * (model, 1) per vertex with Mat4f * Vec4f evaluated as the
// reference's framework writes it (Math.hpp:990-1001: r[i] = sum over j of
// m(i, j) * v[j], accumulated left to right from zero, each operation rounded
// on its own); per-vertex RGBA colours (optional) are copied behind the
// position to form GouraudVertex records. Below it, vertexShader_gouraud and
// vertexShader_texPhong (Shaders.cu:55-108).
#include "cudaraster.h"
#include "cudaraster/ShaderMath.hpp"
#include "cudaraster/detail/device.cuh"
#include "cudaraster/detail/launch.h"

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
    if (!model || !out_vertices || !mvp_row_major || num_vertices < 0 || (num_vertices + 255) / 256 > 0x7FFFFFFF ||
        model_stride < 3 ||
        (out_stride_bytes != 16 && out_stride_bytes != 32) || (colors && color_stride < 4) ||
        ((uintptr_t)out_vertices & 15))
        return CR_ERR_INVALID_ARGUMENT;
    if (num_vertices == 0) return CR_OK;
    cr::Mvp m;
    for (int k = 0; k < 16; k++) m.m[k] = mvp_row_major[k];
    int64_t grid = (num_vertices + 255) / 256;
    const cudaError_t e = cr::launchKernel(cr::vertexPassthroughKernel, (unsigned)grid, 256, 0, (cudaStream_t)stream,
                                           false, model, model_stride, colors, color_stride, (float4*)out_vertices,
                                           out_stride_bytes / 16, num_vertices, m);
    return e == cudaSuccess ? CR_OK : CR_ERR_CUDA;
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

struct GouraudArgs {
    const float* materials;  // records of materialStride floats: diffuse rgba, specular rgb, glossiness, ...
    int materialStride;
    int numMaterials;
    const int* materialIdx;  // one per vertex, clamped to the table
};

enum class VertexKind { Gouraud, TexPhong };

template <VertexKind K>
struct VertexOut {
    static constexpr int kF4 = K == VertexKind::Gouraud ? 2 : 4;  // float4s per output record
};

// One vertex: its InputVertex record (Shaders.hpp: modelPos, modelNormal,
// texCoord; 8 floats) -> a GouraudVertex record (clipPos, lit colour with the
// diffuse alpha) or a ShadedVertex_texPhong record (clipPos, cameraPos,
// cameraNormal with w 0, texCoord with z 0 and w 1).
template <VertexKind K>
__device__ __forceinline__ void shadeVertex(const F32 v[8], int64_t i, const VertexConstants& c, const GouraudArgs& g,
                                            float4* o) {
    const F32 pos[4] = {v[0], v[1], v[2], 1.0f};
    const F32 nrm[3] = {v[3], v[4], v[5]};
    if constexpr (K == VertexKind::Gouraud) {
        F32 cameraPos[3], cameraNormal[3], clip[4];
        matVec<3, 4>(c.posToCamera, pos, cameraPos);
        matVec<3, 3>(c.normalToCamera, nrm, cameraNormal);
        matVec<4, 4>(c.posToClip, pos, clip);
        const int mi = min(max(__ldg(g.materialIdx + i), 0), g.numMaterials - 1);
        const float* mat = g.materials + (int64_t)mi * g.materialStride;
        const FW::Vec3f color = FW::evaluateLighting(
            FW::Vec3f(cameraPos[0], cameraPos[1], cameraPos[2]),
            FW::Vec3f(cameraNormal[0], cameraNormal[1], cameraNormal[2]),
            FW::Vec3f(__ldg(mat + 4), __ldg(mat + 5), __ldg(mat + 6)), __ldg(mat + 7),
            FW::Vec3f(__ldg(mat + 0), __ldg(mat + 1), __ldg(mat + 2)));
        o[0] = make_float4(clip[0], clip[1], clip[2], clip[3]);
        o[1] = make_float4(color.x, color.y, color.z, __ldg(mat + 3));
    } else {
        F32 clip[4], cameraPos[4], cameraNormal[3];
        matVec<4, 4>(c.posToClip, pos, clip);
        matVec<4, 4>(c.posToCamera, pos, cameraPos);
        matVec<3, 3>(c.normalToCamera, nrm, cameraNormal);
        o[0] = make_float4(clip[0], clip[1], clip[2], clip[3]);
        o[1] = make_float4(cameraPos[0], cameraPos[1], cameraPos[2], cameraPos[3]);
        o[2] = make_float4(cameraNormal[0], cameraNormal[1], cameraNormal[2], 0.0f);
        o[3] = make_float4(v[6], v[7], 0.0f, 1.0f);
    }
}

// Records only 4-byte aligned: each thread reads its own record with scalar loads.
template <VertexKind K>
__global__ void __launch_bounds__(256) vertexKernel(const float* __restrict__ in, int64_t n, VertexConstants c,
                                                    GouraudArgs g, float4* __restrict__ out) {
    constexpr int F = VertexOut<K>::kF4;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    F32 v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = __ldg(in + i * 8 + k);
    float4 o[F];
    shadeVertex<K>(v, i, c, g, o);
#pragma unroll
    for (int k = 0; k < F; k++) out[i * F + k] = o[k];
}

// Records 16-byte aligned: the block's 256 input and output records pass
// through shared memory, so every global load and store is a coalesced
// 16-byte access. Used for the texPhong shader, whose 64-byte records make it
// store-bound (0.347 -> 0.318 ms on 16.7M vertices); the Gouraud shader's
// lighting is compute-heavy, and there the staged block's separate load,
// compute and store phases measured slower (0.225 -> 0.323 ms) than threads
// that overlap them freely.
template <VertexKind K>
__global__ void __launch_bounds__(256) vertexKernelStaged(const float4* __restrict__ in, int64_t n, VertexConstants c,
                                                          GouraudArgs g, float4* __restrict__ out) {
    constexpr int F = VertexOut<K>::kF4;
    __shared__ float4 sIn[256 * 2];
    __shared__ float4 sOut[256 * F];
    const int64_t base = (int64_t)blockIdx.x * 256;
    const int cnt = (int)min((int64_t)256, n - base);  // >= 1: the grid covers n exactly
    for (int k = threadIdx.x; k < cnt * 2; k += 256) sIn[k] = __ldg(in + base * 2 + k);
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
        const float4 a = sIn[threadIdx.x * 2], b = sIn[threadIdx.x * 2 + 1];
        const F32 v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        float4 o[F];
        shadeVertex<K>(v, base + threadIdx.x, c, g, o);
#pragma unroll
        for (int k = 0; k < F; k++) sOut[threadIdx.x * F + k] = o[k];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < cnt * F; k += 256) out[base * F + k] = sOut[k];
}

template <VertexKind K>
static cr_status launchVertex(const void* in, int64_t n, const VertexConstants& c, const GouraudArgs& g, void* out,
                              cudaStream_t stream) {
    const unsigned grid = (unsigned)((n + 255) / 256);
    cudaError_t e;
    if (K == VertexKind::TexPhong && ((uintptr_t)in & 15) == 0)
        e = launchKernel(vertexKernelStaged<K>, grid, 256, 0, stream, false, (const float4*)in, n, c, g, (float4*)out);
    else
        e = launchKernel(vertexKernel<K>, grid, 256, 0, stream, false, (const float*)in, n, c, g, (float4*)out);
    return e == cudaSuccess ? CR_OK : CR_ERR_CUDA;
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
    const cr::GouraudArgs g{(const float*)materials, material_stride_bytes / 4, num_materials, vertex_material_idx};
    return cr::launchVertex<cr::VertexKind::Gouraud>(in_vertices, num_vertices, cr::toConstants(constants), g,
                                                     out_vertices, (cudaStream_t)stream);
}

extern "C" cr_status cr_vertex_shader_tex_phong(const void* in_vertices, int64_t num_vertices,
                                               const cr_vertex_constants* constants, void* out_vertices,
                                               void* stream) {
    if (!in_vertices || !constants || !out_vertices || num_vertices < 0 || !cr::gridFits(num_vertices) ||
        ((uintptr_t)out_vertices & 15) || ((uintptr_t)in_vertices & 3))
        return CR_ERR_INVALID_ARGUMENT;
    if (num_vertices == 0) return CR_OK;
    const cr::GouraudArgs g{nullptr, 0, 0, nullptr};
    return cr::launchVertex<cr::VertexKind::TexPhong>(in_vertices, num_vertices, cr::toConstants(constants), g,
                                                      out_vertices, (cudaStream_t)stream);
}

extern "C" cr_status cr_pow_exact(const float* x, const float* y, float* out, int64_t n, void* stream) {
    if (!x || !y || !out || n < 0 || !cr::gridFits(n)) return CR_ERR_INVALID_ARGUMENT;
    if (n == 0) return CR_OK;
    const cudaError_t e = cr::launchKernel(cr::powExactKernel, (unsigned)((n + 255) / 256), 256, 0,
                                           (cudaStream_t)stream, false, x, y, out, n);
    return e == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}
