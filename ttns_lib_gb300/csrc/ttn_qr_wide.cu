// QR of tall matrices wider than the cooperative kernels take (kQrMaxCols < n <=
// kMaxBond): bonds that subspace expansion grows past 64.  The factorisation is
// cuSOLVER's zgeqrf / zungqr (LAPACK conventions: zlarfg reflectors with a real diagonal
// of R, beta = -sign(Re alpha) |x|, tau = 0 for a zero column -- the same gauge as the
// cooperative kernels and the oracle), on a column-major copy: the row-major m x n node
// matrix is transposed by the r2l permutation kernel, factorised, R is read from the
// upper triangle before zungqr overwrites it with Q, and Q is transposed back.
//
// cuSOLVER is loaded on first use (dlopen), not linked: the library and its callers that
// never grow a bond past 64 do not depend on it, and a missing cuSOLVER fails only the
// wide-bond integrators, with an error.
#include "ttn_kernels.cuh"

#include <dlfcn.h>

#include <algorithm>
#include <mutex>
#include <vector>

namespace ttn {

namespace {

// the cuSOLVER dense entry points used here (status 0 is success; cuDoubleComplex has the
// layout of double2)
struct Solver {
  int (*create)(void**) = nullptr;
  int (*destroy)(void*) = nullptr;
  int (*set_stream)(void*, cudaStream_t) = nullptr;
  int (*geqrf_bs)(void*, int, int, double2*, int, int*) = nullptr;
  int (*geqrf)(void*, int, int, double2*, int, double2*, double2*, int, int*) = nullptr;
  int (*ungqr_bs)(void*, int, int, int, const double2*, int, const double2*, int*) = nullptr;
  int (*ungqr)(void*, int, int, int, double2*, int, const double2*, double2*, int, int*) = nullptr;
  bool ok = false;
};

const Solver& solver() {
  static Solver S;
  static std::once_flag once;
  std::call_once(once, [] {
    void* h = nullptr;
    for (const char* name : {"libcusolver.so.12", "libcusolver.so.13", "libcusolver.so.11", "libcusolver.so"})
      if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) return;
    S.create = reinterpret_cast<int (*)(void**)>(dlsym(h, "cusolverDnCreate"));
    S.destroy = reinterpret_cast<int (*)(void*)>(dlsym(h, "cusolverDnDestroy"));
    S.set_stream = reinterpret_cast<int (*)(void*, cudaStream_t)>(dlsym(h, "cusolverDnSetStream"));
    S.geqrf_bs = reinterpret_cast<int (*)(void*, int, int, double2*, int, int*)>(dlsym(h, "cusolverDnZgeqrf_bufferSize"));
    S.geqrf = reinterpret_cast<int (*)(void*, int, int, double2*, int, double2*, double2*, int, int*)>(
        dlsym(h, "cusolverDnZgeqrf"));
    S.ungqr_bs = reinterpret_cast<int (*)(void*, int, int, int, const double2*, int, const double2*, int*)>(
        dlsym(h, "cusolverDnZungqr_bufferSize"));
    S.ungqr = reinterpret_cast<int (*)(void*, int, int, int, double2*, int, const double2*, double2*, int, int*)>(
        dlsym(h, "cusolverDnZungqr"));
    S.ok = S.create && S.destroy && S.set_stream && S.geqrf_bs && S.geqrf && S.ungqr_bs && S.ungqr;
  });
  return S;
}

}  // namespace

struct WideQr {
  void* h = nullptr;
  double2* colmaj = nullptr;  // m x n column-major copy, then Q
  double2* tau = nullptr;     // n reflector scalars
  double2* work = nullptr;    // LAPACK workspace
  int* info = nullptr;
  int lwork = 0;
  long long max_elems = 0;
  int max_n = 0;
};

namespace {

__global__ void k_upper_r(const double2* __restrict__ F, long long m, int n, double2* __restrict__ R, int Rt) {
  const long long total = (long long)n * n;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    const double2 v = (i <= j) ? F[(long long)j * m + i] : make_double2(0.0, 0.0);
    R[Rt ? (long long)j * n + i : e] = v;
  }
}

cudaError_t status_to_cuda(int s) { return s == 0 ? cudaSuccess : cudaErrorUnknown; }

cudaError_t lwork_for(void* h, long long m, int n, double2* A, double2* tau, int* lw) {
  const Solver& S = solver();
  int a = 0, b = 0;
  int s = S.geqrf_bs(h, (int)m, n, A, (int)m, &a);
  if (s != 0) return status_to_cuda(s);
  s = S.ungqr_bs(h, (int)m, n, n, A, (int)m, tau, &b);
  if (s != 0) return status_to_cuda(s);
  *lw = std::max(a, b);
  return cudaSuccess;
}

}  // namespace

cudaError_t wide_qr_create(WideQr** out, const long long* ms, const int* ns, int nshapes, cudaStream_t s) {
  *out = nullptr;
  WideQr* q = new WideQr();
  auto fail = [&](cudaError_t e) { wide_qr_destroy(q); return e; };
  for (int k = 0; k < nshapes; ++k) {
    if (ns[k] < 1 || ns[k] > kMaxBond || ms[k] < ns[k] || ms[k] > 0x7fffffffLL) return fail(cudaErrorInvalidValue);
    q->max_elems = std::max(q->max_elems, ms[k] * ns[k]);
    q->max_n = std::max(q->max_n, ns[k]);
  }
  if (q->max_n == 0) return fail(cudaErrorInvalidValue);
  const Solver& S = solver();
  if (!S.ok) return fail(cudaErrorSharedObjectInitFailed);  // cuSOLVER not found
  if (S.create(&q->h) != 0) return fail(cudaErrorUnknown);
  if (S.set_stream(q->h, s) != 0) return fail(cudaErrorUnknown);
  cudaError_t e;
  if ((e = cudaMalloc(&q->colmaj, (size_t)q->max_elems * sizeof(double2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&q->tau, (size_t)q->max_n * sizeof(double2))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&q->info, sizeof(int))) != cudaSuccess) return fail(e);
  int lw = 1;
  for (int k = 0; k < nshapes; ++k) {
    int l = 0;
    if ((e = lwork_for(q->h, ms[k], ns[k], q->colmaj, q->tau, &l)) != cudaSuccess) return fail(e);
    lw = std::max(lw, l);
  }
  q->lwork = lw;
  if ((e = cudaMalloc(&q->work, (size_t)lw * sizeof(double2))) != cudaSuccess) return fail(e);
  *out = q;
  return cudaSuccess;
}

void wide_qr_destroy(WideQr* q) {
  if (!q) return;
  if (q->work) cudaFree(q->work);
  if (q->info) cudaFree(q->info);
  if (q->tau) cudaFree(q->tau);
  if (q->colmaj) cudaFree(q->colmaj);
  if (q->h) solver().destroy(q->h);
  delete q;
}

cudaError_t householder_qr_wide(WideQr* q, double2* M, long long m, int n, double2* R, int Rt, cudaStream_t s) {
  if (!q || n < 1 || n > q->max_n || m < n || m * n > q->max_elems || m > 0x7fffffffLL) return cudaErrorInvalidValue;
  int need = 0;
  cudaError_t e = lwork_for(q->h, m, n, q->colmaj, q->tau, &need);
  if (e != cudaSuccess) return e;
  if (need > q->lwork) return cudaErrorInvalidValue;
  const Solver& S = solver();
  if (S.set_stream(q->h, s) != 0) return cudaErrorUnknown;
  // row-major m x n -> column-major (the transpose, row-major n x m)
  permute_mode_last(M, q->colmaj, 1, (int)m, n, s);
  e = status_to_cuda(S.geqrf(q->h, (int)m, n, q->colmaj, (int)m, q->tau, q->work, q->lwork, q->info));
  if (e != cudaSuccess) return e;
  const long long nn = (long long)n * n;
  const int blocks = (int)std::min<long long>((nn + 255) / 256, 1024);
  k_upper_r<<<blocks, 256, 0, s>>>(q->colmaj, m, n, R, Rt);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  e = status_to_cuda(S.ungqr(q->h, (int)m, n, n, q->colmaj, (int)m, q->tau, q->work, q->lwork, q->info));
  if (e != cudaSuccess) return e;
  unpermute_mode_last(q->colmaj, M, 1, (int)m, n, s);
  return cudaGetLastError();
}

}  // namespace ttn
