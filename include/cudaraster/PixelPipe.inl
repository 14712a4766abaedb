// PixelPipe.inl -- include from a .cu file to define pixel pipes.
//
//   CR_DEFINE_PIXEL_PIPE(PipeName, ShadedVertexClass, FragmentShaderClass,
//                        BlendShaderClass, SamplesLog2, RenderModeFlags)
//
// Same macro and arguments as the reference (PixelPipe.inl:241-275). It
// instantiates the setup and fine kernels for the pipe and registers the
// pipe under "PipeName" when the object is loaded, with the spec the
// reference kept in PipeName_spec (samples, vertex size, flags, blend shader
// name). The bin and coarse stages do not depend on the pipe and live in the
// runtime library.
#pragma once

#include "PixelPipe.hpp"
#include "detail/fine.cuh"
#include "detail/per_device.h"
#include "detail/pipe_registry.h"
#include "detail/setup.cuh"

#include <string.h>

#ifndef CR_PROFILING_MODE
#define CR_PROFILING_MODE ProfilingMode_Default
#endif

namespace cr {

template <class V, class FS, class BS, int S, uint32_t F>
struct PipeImpl {
    static_assert(sizeof(V) % 16 == 0 && sizeof(V) >= 16, "vertex struct must be Vec4f records");
    static_assert(S >= 0 && S <= 3, "SamplesLog2 must be 0..3");

    static cudaError_t launchSetup(const DrawDev& d, int instBegin, int instEnd, int64_t triBegin, int64_t triEnd,
                                   cudaStream_t stream) {
        int64_t n = triEnd - triBegin;
        if (n <= 0) return cudaSuccess;
        unsigned grid = (unsigned)((n + 255) / 256);
        return launchKernel(setupKernel<S, F & (kRenderDepth | kRenderLerp)>, grid, 256, 0, stream, true, d, instBegin,
                            instEnd, (S64)triBegin, (S64)triEnd);
    }
    static size_t smemBytes(int warps) { return sizeof(typename FineTraits<FS, BS, S, F>::Smem) * (size_t)warps; }
    static cudaError_t launchFine(const DrawDev& d, int group, int32_t tileBegin, int32_t tileEnd, int warps,
                                  int ctasPerSM, int numSMs, cudaStream_t stream) {
        if (tileEnd <= tileBegin) return cudaSuccess;
        auto kern = fineKernelFor<V, FS, BS, S, F>();
        configureFine();
        int64_t warpsNeeded = tileEnd - tileBegin;
        int64_t grid = (int64_t)numSMs * ctasPerSM;
        int64_t maxGrid = (warpsNeeded + warps - 1) / warps;
        if (grid > maxGrid) grid = maxGrid;
        if (grid < 1) grid = 1;
        return launchKernel(kern, (unsigned)grid, warps * 32, smemBytes(warps), stream, true, d, group, tileBegin,
                            tileEnd);
    }
    // The fine kernel's shared-memory limit, set once on each device used.
    static void configureFine() {
        static OncePerDevice once;
        once.run([] {
            cudaFuncSetAttribute(fineKernelFor<V, FS, BS, S, F>(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 160 * 1024);
        });
    }
    // Resident fine CTAs per SM, by warps per CTA (queried once per size and device).
    static int fineOccupancy(int warps) {
        static IntsPerDevice<9> cache;
        const int w = warps >= 1 && warps <= 8 ? warps : 8;
        configureFine();
        return cache.get(w, [](int ww) {
            int blocks = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fineKernelFor<V, FS, BS, S, F>(), ww * 32,
                                                              smemBytes(ww)) != cudaSuccess)
                return 1;
            return blocks > 0 ? blocks : 1;
        });
    }
    static void describe(PipeDesc& p, const char* name, const char* blend, const char* frag) {
        memset(&p, 0, sizeof(p));
        strncpy(p.name, name, sizeof(p.name) - 1);
        strncpy(p.blendShaderName, blend, sizeof(p.blendShaderName) - 1);
        strncpy(p.fragmentShaderName, frag, sizeof(p.fragmentShaderName) - 1);
        p.samplesLog2 = S;
        p.vertexStructSize = (int32_t)sizeof(V);
        p.renderModeFlags = F;
        p.profilingMode = CR_PROFILING_MODE;
        p.launchSetup = &launchSetup;
        p.launchFine = &launchFine;
        p.fineOccupancy = &fineOccupancy;
    }
};

}  // namespace cr

#define CR_DEFINE_PIXEL_PIPE(PIPE_NAME, VERTEX_STRUCT, FRAGMENT_SHADER, BLEND_SHADER, SAMPLES_LOG2, RENDER_MODE_FLAGS) \
    namespace {                                                                                                         \
    struct PIPE_NAME##_registrar {                                                                                      \
        PIPE_NAME##_registrar() {                                                                                       \
            cr::PipeDesc desc;                                                                                          \
            cr::PipeImpl<VERTEX_STRUCT, FRAGMENT_SHADER, BLEND_SHADER, (SAMPLES_LOG2), (uint32_t)(RENDER_MODE_FLAGS)>:: \
                describe(desc, #PIPE_NAME, #BLEND_SHADER, #FRAGMENT_SHADER);                                            \
            cr_register_pipe(&desc);                                                                                    \
        }                                                                                                               \
    };                                                                                                                  \
    PIPE_NAME##_registrar PIPE_NAME##_registrar_instance;                                                               \
    }
