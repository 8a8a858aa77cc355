// Programmatic dependent launch: a kernel of the evaluation sequence lets the next one
// launch as soon as all of its own blocks have started, and waits for the whole previous
// grid (including its memory operations) before touching anything.  Both instructions
// are no-ops when a kernel was launched without the programmatic attribute.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace nnapgb {

__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch with the programmatic-stream-serialization attribute (captured into CUDA graphs
// as a programmatic dependency).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace nnapgb
