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
