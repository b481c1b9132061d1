// Tensor-core (tcgen05) contractions for the mixed-precision form.
//
// Complex products are done as real GEMMs in the block form
//     [Re; Im](S v) = [[Sr, -Si], [Si, Sr]] [Re v; Im v],
// operands split as x = hi + lo in TF32 and the products accumulated in FP32 in two TMEM
// accumulators, hi*hi and hi*lo + lo*hi, summed at the end (the error-compensated TF32
// scheme of Ootomo & Yokota, IJHPCA 2022).  Inputs and outputs stay complex128 in HBM.
#include "ttn_tc.cuh"
#include "ttn_tc_core.cuh"
#include "ttn_kernels.cuh"


namespace ttn {

using namespace tc;

namespace {
constexpr int kTcSmem = 232448 - 2048;  // the dynamic shared memory a CTA may hold next to its static part

// D (128 x N) = A (128 x K) * B (N x K)^T for one CTA; fp64 in and out.
__global__ void __launch_bounds__(256) k_tc_gemm_test(const double* __restrict__ A, const double* __restrict__ B,
                                                     double* __restrict__ D, int K, int N, int* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t* a_hi = (uint32_t*)smem;
  uint32_t* a_lo = a_hi + 128 * K;
  uint32_t* b_hi = a_lo + 128 * K;
  uint32_t* b_lo = b_hi + N * K;
  for (int e = threadIdx.x; e < 128 * K; e += blockDim.x) {
    const int row = e / K, k = e % K;
    uint32_t h, l;
    split_tf32(A[e], h, l);
    a_hi[tf32_offset(row, k, 128) / 4] = h;
    a_lo[tf32_offset(row, k, 128) / 4] = l;
  }
  for (int e = threadIdx.x; e < N * K; e += blockDim.x) {
    const int row = e / K, k = e % K;
    uint32_t h, l;
    split_tf32(B[e], h, l);
    b_hi[tf32_offset(row, k, N) / 4] = h;
    b_lo[tf32_offset(row, k, N) / 4] = l;
  }
  if (threadIdx.x == 0) mbar_init(&mbar, 1);
  if (warp == 0) tmem_alloc(&tmem_base, 128);
  fence_proxy_async();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tm = tmem_base;
  if (threadIdx.x == 0) {
    const uint32_t idesc = idesc_tf32(128, N);
    const uint32_t lboA = (128 / 8) * 128, lboB = (uint32_t)(N / 8) * 128, sbo = 128;
    for (int kk = 0; kk < K / 8; ++kk) {
      const uint32_t offA = (uint32_t)kk * 2 * (128 / 8) * 128, offB = (uint32_t)kk * 2 * (N / 8) * 128;
      const uint64_t ah = smem_desc(smem_u32(a_hi) + offA, lboA, sbo), al = smem_desc(smem_u32(a_lo) + offA, lboA, sbo);
      const uint64_t bh = smem_desc(smem_u32(b_hi) + offB, lboB, sbo), bl = smem_desc(smem_u32(b_lo) + offB, lboB, sbo);
      mma_tf32(tm, ah, bh, idesc, kk > 0);
      mma_tf32(tm + N, ah, bl, idesc, kk > 0);
      mma_tf32(tm + N, al, bh, idesc, 1);
    }
    mma_commit(&mbar);
  }
  __syncwarp();
  if (!mbar_wait(&mbar, 0) && lane == 0) atomicOr(err, kErrMmaTimeout);
  fence_after();
  if (warp < 4) {
    const int row = 32 * warp + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
      float mv[16], cv[16];
      tmem_ld16(tm + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, mv);
      tmem_ld16(tm + ((uint32_t)(32 * warp) << 16) + (uint32_t)(N + c0), cv);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[(long long)row * N + c0 + i] = (double)mv[i] + (double)cv[i];
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tm, 128);
  }
}
}  // namespace

cudaError_t tc_gemm_test(const double* A, const double* B, double* D, int K, int N, int* err, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(k_tc_gemm_test, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  if (e != cudaSuccess) return e;
  ++g_launches;
  k_tc_gemm_test<<<1, 256, kTcSmem, s>>>(A, B, D, K, N, err);
  return cudaGetLastError();
}

}  // namespace ttn
