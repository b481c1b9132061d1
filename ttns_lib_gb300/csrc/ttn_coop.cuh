// Grid-wide cooperation primitives for the persistent kernels (QR, Krylov).
#pragma once
#include <cuda_runtime.h>

namespace ttn {

// Status bits written by device code (never a trap).
enum : int {
  kErrNonFinite = 1,          // non-finite values in the state after a step
  kKrylovErrShift = 2,        // Krylov error bits (reject limit, non-finite, eigen-solve, step, sub-step limit) << 2
  kErrBarrierTimeout = 1 << 12
};

// Barrier state in device memory: {count, generation}; zero-initialised once.
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
};

#ifdef __CUDACC__
// Sense-reversing grid barrier with a bounded wait.  Requires a cooperative launch
// (all blocks co-resident).  On timeout it sets kErrBarrierTimeout in *err and every
// later barrier returns at once, so the kernel runs to completion and the host sees
// the error instead of a hung device.
__device__ __forceinline__ void grid_barrier(GridBarrier* b, int* err) {
  if (gridDim.x == 1) {  // one CTA: the block barrier orders its global accesses already
    __syncthreads();
    return;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = &b->gen;
    const unsigned int g = *vgen;
    __threadfence();
    const unsigned int arrived = atomicAdd(&b->count, 1u);
    if (arrived == gridDim.x - 1) {
      b->count = 0;
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      unsigned long long it = 0;
      while (*vgen == g) {
        if (*(volatile int*)err & kErrBarrierTimeout) break;
        if (++it > (1ull << 26)) {
          atomicOr(err, kErrBarrierTimeout);
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
}
#endif  // __CUDACC__

}  // namespace ttn
