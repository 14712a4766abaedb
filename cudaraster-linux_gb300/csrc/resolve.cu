// resolve.cu -- MSAA resolve of a colour surface into a linear RGBA8 image.
//
// The reference's resolve (CudaSurface::resolveToScreen, CudaSurface.hpp:73)
// is commented out and would have drawn through GL. Here one thread per
// pixel averages the pixel's samples channel by channel, rounding half up:
// c = (sum of the S samples' channel + S/2) >> log2 S, and writes the pixel
// to a row-major image (one 32-bit word per pixel, R in the low byte as the
// surface words are). With one sample it only drops the 8x8 tile padding.
#include <cuda_runtime.h>

#include <cstdint>

#include "cudaraster.h"

namespace cr {
namespace {

__global__ void resolveKernel(const uint32_t* __restrict__ color, int width, int height, int samplesLog2,
                              int64_t rowWords, uint32_t* __restrict__ out, int64_t outRowWords) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= width || y >= height) return;
    const int ns = 1 << samplesLog2;
    const int64_t base = (int64_t)y * rowWords + (int64_t)(x >> 3) * 8 * ns + (x & 7);
    uint32_t sum[4] = {0, 0, 0, 0};
    for (int i = 0; i < ns; i++) {
        const uint32_t c = color[base + i * 8];
#pragma unroll
        for (int k = 0; k < 4; k++) sum[k] += (c >> (8 * k)) & 0xFFu;
    }
    uint32_t px = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) px |= ((sum[k] + (uint32_t)(ns >> 1)) >> samplesLog2) << (8 * k);
    out[(int64_t)y * outRowWords + x] = px;
}

}  // namespace
}  // namespace cr

extern "C" cr_status cr_resolve_color(const void* color, int32_t width, int32_t height, int32_t num_samples, void* out,
                                      int64_t out_row_bytes, void* stream) {
    if (!color || !out || width <= 0 || height <= 0 || width > CR_MAX_VIEWPORT || height > CR_MAX_VIEWPORT ||
        num_samples < 1 || num_samples > 8 || (num_samples & (num_samples - 1)) || out_row_bytes < (int64_t)width * 4 ||
        (out_row_bytes & 3))
        return CR_ERR_INVALID_ARGUMENT;
    int log2 = 0;
    while ((1 << log2) < num_samples) log2++;
    const int64_t rowWords = (int64_t)((width + 7) & ~7) * num_samples;
    const dim3 block(32, 8), grid((width + 31) / 32, (height + 7) / 8);
    cr::resolveKernel<<<grid, block, 0, (cudaStream_t)stream>>>((const uint32_t*)color, width, height, log2, rowWords,
                                                               (uint32_t*)out, out_row_bytes / 4);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}
