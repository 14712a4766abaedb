// texture.cu -- the textured pipe's atlas filter (crTex2D) over arrays, and
// the same lookups through the GPU's texture unit. The second exists to
// compare the specified filter with the hardware filter the reference's
// tex2D used (linear filtering, wrap addressing, normalized coordinates on an
// RGBA8 array read as normalized floats); it is not used by any pipe.
#include "cudaraster.h"
#include "cudaraster/ShaderMath.hpp"
#include "cudaraster/detail/device.cuh"
#include "cudaraster/detail/launch.h"

namespace cr {

__global__ void __launch_bounds__(256) textureSampleKernel(FW::TextureAtlas atlas, const float2* __restrict__ uv,
                                                           float4* __restrict__ out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 p = uv[i];
    const FW::Vec4f c = FW::crTex2D(atlas, p.x, p.y);
    out[i] = make_float4(c.x, c.y, c.z, c.w);
}

__global__ void __launch_bounds__(256) textureSampleHwKernel(cudaTextureObject_t tex, const float2* __restrict__ uv,
                                                             float4* __restrict__ out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 p = uv[i];
    out[i] = tex2D<float4>(tex, p.x, p.y);
}

static bool validSample(const uint32_t* atlas, int32_t w, int32_t h, const float* uv, const float* out, int64_t n) {
    return atlas && uv && out && w >= 1 && h >= 1 && w <= 65536 && h <= 65536 && n >= 0 &&
           (n + 255) / 256 <= 0x7FFFFFFF && !((uintptr_t)atlas & 3) && !((uintptr_t)uv & 7) && !((uintptr_t)out & 15);
}

}  // namespace cr

extern "C" cr_status cr_texture_sample(const uint32_t* atlas, int32_t atlas_width, int32_t atlas_height,
                                       const float* uv, float* out, int64_t n, void* stream) {
    if (!cr::validSample(atlas, atlas_width, atlas_height, uv, out, n)) return CR_ERR_INVALID_ARGUMENT;
    if (n == 0) return CR_OK;
    const cudaError_t e = cr::launchKernel(cr::textureSampleKernel, (unsigned)((n + 255) / 256), 256, 0,
                                           (cudaStream_t)stream, false, FW::TextureAtlas{atlas, atlas_width, atlas_height},
                                           (const float2*)uv, (float4*)out, n);
    return e == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

extern "C" cr_status cr_texture_sample_hw(const uint32_t* atlas, int32_t atlas_width, int32_t atlas_height,
                                          const float* uv, float* out, int64_t n, void* stream) {
    if (!cr::validSample(atlas, atlas_width, atlas_height, uv, out, n)) return CR_ERR_INVALID_ARGUMENT;
    if (n == 0) return CR_OK;
    const cudaStream_t s = (cudaStream_t)stream;
    cudaChannelFormatDesc fmt = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsigned);
    cudaArray_t array = nullptr;
    if (cudaMallocArray(&array, &fmt, (size_t)atlas_width, (size_t)atlas_height) != cudaSuccess)
        return CR_ERR_OUT_OF_MEMORY;
    cudaTextureObject_t tex = 0;
    cudaError_t e = cudaMemcpy2DToArrayAsync(array, 0, 0, atlas, (size_t)atlas_width * 4, (size_t)atlas_width * 4,
                                             (size_t)atlas_height, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) {
        cudaResourceDesc res = {};
        res.resType = cudaResourceTypeArray;
        res.res.array.array = array;
        cudaTextureDesc td = {};
        td.addressMode[0] = cudaAddressModeWrap;
        td.addressMode[1] = cudaAddressModeWrap;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeNormalizedFloat;
        td.normalizedCoords = 1;
        e = cudaCreateTextureObject(&tex, &res, &td, nullptr);
    }
    if (e == cudaSuccess) {
        e = cr::launchKernel(cr::textureSampleHwKernel, (unsigned)((n + 255) / 256), 256, 0, s, false, tex,
                             (const float2*)uv, (float4*)out, n);
    }
    const cudaError_t es = cudaStreamSynchronize(s);
    if (tex) cudaDestroyTextureObject(tex);
    cudaFreeArray(array);
    return e == cudaSuccess && es == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}
