// Stand-alone check of the tcgen05 building blocks (TMEM, shared-memory descriptors, MMA
// issue, commit and bounded mbarrier waits) used by the sweep's tensor-core contractions.
#pragma once
#include <cuda_runtime.h>

namespace ttn {

// One-CTA check of the tcgen05 path: D (128 x N) = A (128 x K) * B (N x K)^T, fp64 in/out,
// split-TF32 products with FP32 accumulation.  N in {16, 32, ..., 256}, K a multiple of 8,
// 2*(128+N)*K*4 bytes of operands must fit in shared memory.
cudaError_t tc_gemm_test(const double* A, const double* B, double* D, int K, int N, int* err, cudaStream_t s);

}  // namespace ttn
