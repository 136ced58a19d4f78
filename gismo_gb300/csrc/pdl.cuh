// Programmatic dependent launch: a kernel launched with the programmatic-serialization attribute
// may be scheduled before the kernel it follows has finished; it calls pdlWait() before touching
// anything that kernel writes (the wait returns once the preceding grid has completed and its
// memory is visible), and the preceding kernel calls pdlTrigger() once its blocks are past their
// main work, so the next launch's set-up overlaps its tail. Without the attribute both are no-ops.
#pragma once

#include <cuda_runtime.h>

namespace gsgpu {

__device__ __forceinline__ void pdlWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdlTrigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// launch `kernel` on `s`, with the programmatic-serialization attribute when `pdl` is set
template <typename... KArgs, typename... Args>
inline void launchMaybePdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, bool pdl, Args... args) {
    if (!pdl) {
        kernel<<<grid, block, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, KArgs(args)...);
}

}  // namespace gsgpu
