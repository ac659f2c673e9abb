// Programmatic dependent launch for the explicit time loop's chain of small launches
// (strain row write -> step -> probe read -> ...).
//
// A kernel launched with launch_chained() may be scheduled before its predecessor in the
// stream has finished: as soon as every CTA of the predecessor has executed
// chain_release() (or exited).  Its CTAs then wait in chain_acquire() -- a hardware wait
// for the predecessor's completion and the visibility of all its memory operations -- and
// start at once when it ends, instead of after a full launch round trip.
//
// Rules that keep this correct:
//  - every kernel launched with launch_chained() calls chain_acquire() before its first
//    access to global memory;
//  - chain_release() only lets the successor be scheduled: the successor still waits for
//    this grid's completion in its own chain_acquire().  Because the successor is
//    scheduled only after every CTA of this grid has been scheduled and released, its CTAs
//    never hold the resources this grid still needs.
#pragma once
#include <cuda_runtime.h>

#include <utility>

namespace nrt {

__device__ __forceinline__ void chain_acquire() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ void chain_release() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Adds n to the count of kernels this library has launched (nrt_kernel_launches; api.cu).
void count_launches(long long n);

// Counts one launch on st unless st is being captured into a graph (a replay of the graph
// counts its kernel nodes then).
inline void count_launch_on(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone)
    count_launches(1);
}

template <typename... KArgs, typename... Args>
cudaError_t launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                           cudaStream_t st, Args &&...args) {
  count_launch_on(st);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace nrt
