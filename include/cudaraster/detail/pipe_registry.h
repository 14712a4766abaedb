// pipe_registry.h -- the contract between compiled pixel pipes and the
// runtime. CR_DEFINE_PIXEL_PIPE (PixelPipe.inl) fills one PipeDesc per pipe
// and registers it when its shared object is loaded; cr_set_pixel_pipe()
// looks pipes up by name. This replaces the reference's run-time nvcc
// compile and module/kernel lookup (CudaCompiler.cpp:506-632,
// CudaRaster.cpp:183-216): pipes are compiled ahead of time for sm_103a.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace cr {
struct DrawDev;

struct PipeDesc {
    char name[64];
    int32_t samplesLog2;
    int32_t vertexStructSize;
    uint32_t renderModeFlags;
    int32_t profilingMode;
    char blendShaderName[64];
    char fragmentShaderName[64];
    // Launch the setup kernel over triangles [triBegin, triEnd) of instances
    // [instBegin, instEnd).
    cudaError_t (*launchSetup)(const DrawDev& d, int instBegin, int instEnd, int64_t triBegin,
                               int64_t triEnd, cudaStream_t stream);
    // Launch the fine kernel (persistent grid) over global tiles [tileBegin, tileEnd).
    cudaError_t (*launchFine)(const DrawDev& d, int group, int32_t tileBegin, int32_t tileEnd,
                              int warps, int ctasPerSM, int numSMs, cudaStream_t stream);
    // Resident CTAs per SM of the fine kernel for a block of `warps` warps.
    int (*fineOccupancy)(int warps);
};
}  // namespace cr

extern "C" void cr_register_pipe(const cr::PipeDesc* desc);
