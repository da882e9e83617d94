// Chains of dependent kernels: programmatic dependent launch.
//
// A kernel launched with launch_dependent may be scheduled while the kernel
// before it in the stream is still draining; it must begin with
// pdl_enter(), which waits until that kernel has completed and its writes
// are visible before anything else runs, so the stream's ordering of
// global-memory effects is unchanged.  What overlaps is the launch and the
// CTAs' start-up with the predecessor's tail.  While the stream is being
// captured into a graph the launch is an ordinary one: with several graphs
// in flight the waiting CTAs would hold SM slots the others could use.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace gi {

// First statement of a kernel launched by launch_dependent (no-ops for an
// ordinary launch): wait for the previous grid, then let the next kernel be
// scheduled as this grid's CTAs finish.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// `dependent` false gives an ordinary launch (for grids of many waves the
// CTAs waiting during the predecessor's last wave cost more than the
// overlap gains: measured on the 2048^2 summed-area tables and the EDT).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent_if(bool dependent, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                       cudaStream_t st, Args&&... args) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;  // unknown: launch ordinarily
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = dependent && cap == cudaStreamCaptureStatusNone ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                    Args&&... args) {
    return launch_dependent_if(true, kernel, grid, block, smem, st, std::forward<Args>(args)...);
}

}  // namespace gi
