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
#include "cudaraster/detail/launch.h"

namespace cr {
namespace {

// One thread per pixel; the sample count is a template parameter so the
// sample loads are unrolled and issued together.
template <int samplesLog2>
__global__ void resolveKernel(const uint32_t* __restrict__ color, int width, int height, int64_t rowWords,
                              uint32_t* __restrict__ out, int64_t outRowWords) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= width || y >= height) return;
    constexpr int ns = 1 << samplesLog2;
    const int64_t base = (int64_t)y * rowWords + (int64_t)(x >> 3) * 8 * ns + (x & 7);
    // Channels R and B summed in the 16-bit lanes of `rb`, G and A in those of
    // `ga`: a lane holds at most 8 * 255 + 4 < 2^16, so lanes never carry into
    // each other, and the bits a right shift moves across a lane boundary are
    // masked off.
    uint32_t rb = 0, ga = 0;
#pragma unroll
    for (int i = 0; i < ns; i++) {
        const uint32_t c = __ldg(&color[base + i * 8]);
        rb += c & 0x00FF00FFu;
        ga += (c >> 8) & 0x00FF00FFu;
    }
    constexpr uint32_t half = (uint32_t)(ns >> 1) * 0x00010001u;
    rb = ((rb + half) >> samplesLog2) & 0x00FF00FFu;
    ga = ((ga + half) >> samplesLog2) & 0x00FF00FFu;
    out[(int64_t)y * outRowWords + x] = rb | (ga << 8);
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
    const uint32_t* c = (const uint32_t*)color;
    uint32_t* o = (uint32_t*)out;
    const cudaStream_t s = (cudaStream_t)stream;
    const int32_t ow = (int32_t)(out_row_bytes / 4);
    cudaError_t e;
    switch (log2) {
    case 0: e = cr::launchKernel(cr::resolveKernel<0>, grid, block, 0, s, false, c, width, height, rowWords, o, ow); break;
    case 1: e = cr::launchKernel(cr::resolveKernel<1>, grid, block, 0, s, false, c, width, height, rowWords, o, ow); break;
    case 2: e = cr::launchKernel(cr::resolveKernel<2>, grid, block, 0, s, false, c, width, height, rowWords, o, ow); break;
    default: e = cr::launchKernel(cr::resolveKernel<3>, grid, block, 0, s, false, c, width, height, rowWords, o, ow); break;
    }
    return e == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}
