// pdl.cuh — programmatic dependent launch for the kernel chains of one operation.
//
// A kernel launched with launch_pdl may be scheduled while the previous kernel on its stream is
// still draining its last wave, so its launch latency and block scheduling overlap that tail.
// Every such kernel calls pdl_wait() before its first global-memory access: the instruction
// returns once the previous grid has completed and its writes are visible, so no data hazard
// (read-after-write or write-after-read on shared scratch) can arise.  pdl_release() lets the
// next kernel in the chain be scheduled early in turn.  Launched without the attribute, both
// instructions are no-ops.
#pragma once
#include <cuda_runtime.h>

namespace pfg {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
inline void launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace pfg
