// Programmatic dependent launch for the kernels of one step. A kernel launched with
// launchAfterPrior starts before the previous kernel of the stream has finished: it first
// waits for that kernel (griddepcontrol.wait returns once the prerequisite grid has
// completed and its writes are visible; at once when there is none) and then lets the next
// kernel of the step be launched (whose blocks are scheduled once every block of this one
// is running, and which waits in turn before reading anything). The step's launch latency
// overlaps the previous kernel instead of following it.
#pragma once

#include <cuda_runtime.h>

namespace chiml {
namespace dev {

__device__ __forceinline__ void waitPriorGrid() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline void launchAfterPrior(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace dev
}  // namespace chiml
