// launch.h -- kernel launches that report their own status, optionally as
// programmatic dependent launches.
//
// cudaLaunchKernelEx returns the status of the launch it makes, so an entry
// point does not pick up (and clear) an error left pending by an unrelated
// earlier call, as cudaGetLastError after a <<<>>> launch would.
//
// With pdl set, the kernel is launched with programmatic stream
// serialization: it may begin while the previous kernel on the stream is
// still running, once every CTA of that kernel has executed pdlTrigger() (or
// exited). Such a kernel must execute pdlWait() -- which returns when the
// previous kernel has completed and its memory operations are visible --
// before it reads or writes anything the previous kernel touches. Every
// pipeline kernel calls pdlWait() before its first global memory access, so
// the overlap is limited to launch and CTA dispatch, and the ordering of the
// stages is unchanged. Without the attribute both calls are no-ops.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace cr {

__device__ __forceinline__ void pdlWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdlTrigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... Params, class... Args>
inline cudaError_t launchKernel(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                                bool pdl, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    if (pdl) {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace cr
