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

// Barrier state in device memory, zero-initialised once: a monotonic arrival counter and
// the count at which the current launch started (its base).  A launch reads the base at
// its start (grid_barrier_begin); the k-th barrier of the launch completes when the count
// reaches base + k * gridDim.x; after its last barrier the launch stores its final count
// as the next launch's base (grid_barrier_end).  One arrival and one acquire poll per CTA
// per barrier (about 1.35 us for 152 CTAs on GB300, against 2.25 us for a
// generation-flag barrier with a second atomic on the critical path).
struct GridBarrier {
  unsigned long long count;
  unsigned long long base;
};

#ifdef __CUDACC__
// per-CTA target of the next barrier (one shared slot per kernel)
__device__ __forceinline__ unsigned long long* grid_barrier_slot() {
  __shared__ unsigned long long s_target;
  return &s_target;
}
// at kernel start, before the first grid_barrier (all threads)
__device__ __forceinline__ void grid_barrier_begin(GridBarrier* b) {
  if (threadIdx.x == 0) *grid_barrier_slot() = *(volatile unsigned long long*)&b->base;
  __syncthreads();
}
// Grid barrier with a bounded wait.  Requires a cooperative launch (all blocks
// co-resident).  On timeout it sets kErrBarrierTimeout in *err and every later barrier
// arrives without waiting, so the kernel runs to completion and the host sees the error
// instead of a hung device; the count stays consistent (every CTA still arrives).
__device__ __forceinline__ void grid_barrier(GridBarrier* b, int* err) {
  if (gridDim.x == 1) {  // one CTA: the block barrier orders its global accesses already
    __syncthreads();
    return;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long* slot = grid_barrier_slot();
    const unsigned long long target = *slot + gridDim.x;
    *slot = target;
    asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(&b->count) : "memory");
    if (!(*(volatile int*)err & kErrBarrierTimeout)) {
      unsigned long long v = 0, it = 0;
      for (;;) {
        asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(&b->count) : "memory");
        if (v >= target) break;
        if (++it > (1ull << 26)) {
          atomicOr(err, kErrBarrierTimeout);
          break;
        }
      }
    }
  }
  __syncthreads();
}
// Warp sum of a complex value, the result in every lane: the first level of the butterfly
// splits the two components between the half-warps (each lane keeps one and adds its
// partner's copy of it), the other four reduce one component, and one shuffle returns the
// other half's component.  Five FP64 additions per lane instead of ten: on GB300 one warp's
// FP64 instruction occupies its sub-partition's FP64 pipe for 64 cycles.
__device__ __forceinline__ double2 warp_sum2(double2 v) {
  const bool hi = (threadIdx.x & 16) != 0;
  double k = (hi ? v.y : v.x) + __shfl_xor_sync(0xffffffffu, hi ? v.x : v.y, 16);
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
  const double other = __shfl_xor_sync(0xffffffffu, k, 16);
  return hi ? make_double2(other, k) : make_double2(k, other);
}
// at kernel end, after the last grid_barrier (all threads may call it)
__device__ __forceinline__ void grid_barrier_end(GridBarrier* b) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && gridDim.x > 1) b->base = *grid_barrier_slot();
}
#endif  // __CUDACC__

}  // namespace ttn
