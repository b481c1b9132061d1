// Tensor-core (tcgen05) contraction engine for the mixed-precision form of the sweep.
// Each entry point returns true when it handled the contraction; the FP64 kernels run
// the contraction otherwise (plain form, or shapes the engine does not take).
#pragma once
#include <cuda_runtime.h>

namespace ttn {

struct TcEngine;

// Throws (via the host error path) when the device cannot run the engine.
TcEngine* tc_create(int device, long long max_node_size, cudaStream_t s);
void tc_destroy(TcEngine* e);

bool tc_mode_apply(TcEngine* e, const double2* S, int d, const double2* in, double2* out, long long na, long long nb,
                   double2 alpha, bool acc, cudaStream_t s);
bool tc_mf_apply(TcEngine* e, const double2* in, const double2* M, int r, long long nx, double2* out, double2 alpha,
                 bool acc, cudaStream_t s);
bool tc_adj_mul(TcEngine* e, const double2* A, const double2* X, long long nx, int r, double2* out, double2 alpha,
                bool acc, cudaStream_t s);
bool tc_mode_contract(TcEngine* e, const double2* A, const double2* T, long long na, int d, long long nb, double2* out,
                      double2 alpha, bool acc, cudaStream_t s);

// One-CTA check of the tcgen05 path: D (128 x N) = A (128 x K) * B (N x K)^T, fp64 in/out,
// split-TF32 products with FP32 accumulation.  N in {16, 32, ..., 256}, K a multiple of 8,
// 2*(128+N)*K*4 bytes of operands must fit in shared memory.
cudaError_t tc_gemm_test(const double* A, const double* B, double* D, int K, int N, int* err, cudaStream_t s);

}  // namespace ttn
