// Internal declarations shared by the host orchestration (ttn_host.cpp) and the
// device code (ttn_kernels.cu, ttn_tc.cu).  Not part of the public C-ABI.
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>

namespace ttn {

// kernel launches issued by this library (atomic: ttn_batch_step launches from several
// host threads)
extern std::atomic<unsigned long long> g_launches;

// Element addressing of a GEMM operand.
//   A(i,k) = p[i*s0 + (k/kdiv)*k1 + (k%kdiv)*k2]        (conj if cj)
//   B(k,j) = p[j*s0 + (k/kdiv)*k1 + (k%kdiv)*k2]        (conj if cj)
// kfast tells the tile loader that consecutive k are contiguous in memory.
struct ZOperand {
  const double2* p;
  long long s0, k1, k2, kdiv;
  int cj;
  int kfast;
};

// C(i,j) at c[i*ci + j*cj]; batch z adds z*bs to every pointer.
struct ZGemm {
  int M, N, K;
  ZOperand A, B;
  double2* C;
  long long ci, cj;
  long long bsA, bsB, bsC;
  int batch;
  double2 alpha, beta;
};

// Workspace needed by zgemm when it splits K (bytes).
size_t zgemm_split_workspace_bytes(int M, int N, int K);
// C = alpha * A*B + beta * C on stream s; `ws` is scratch of the size above (may be
// null when K is short enough that no split happens).
void zgemm(const ZGemm& g, double2* ws, size_t ws_bytes, cudaStream_t s);

// ---- Lanczos / Krylov exponential on the device --------------------------------
// Scalar state of one exponential, resident in device memory.
struct KrylovCtl {
  double alpha[72];      // Lanczos diagonal
  double bet[73];        // Lanczos off-diagonal (bet[j] couples j-1 and j)
  double coef[2 * 72];   // combination coefficients (complex) for y = sum_q c_q V_q
  double beta;           // ||y|| at the start of the current sub-step
  double avnorm;         // ||H V_m||
  double t_now, t_new, t_out, sgn;
  double cf_re, cf_im;   // coefficient of the exponent (e.g. -i)
  double tol;
  int m;                 // Krylov dimension
  int mb;                // dimension actually used (breakdown)
  int k1;                // 2 normally, 0 on breakdown
  int done;              // 1 when t_now >= t_out
  int err;               // nonzero: step-size rejection limit hit or non-finite values
  int substeps;
  long long napps;       // H applications (including the error-estimate one)
};

constexpr int kQrMaxCols = 64;   // widest matrix the cooperative device QR kernels accept
constexpr int kMaxBond = 256;    // widest bond of the FP64 sweep (its gauge QRs: ttn_qr_rows.cu, ttn_qr.cu)
constexpr int kKrylovMax = 64;   // largest Krylov dimension

// ---- Householder QR --------------------------------------------------------------
// In-place Householder QR of an m x n row-major matrix (m >= n): M <- Q, R (n x n) out;
// Rt != 0 stores R^T instead of R.  Column-by-column cooperative multi-CTA version
// (grid <= co-resident CTAs); scratch of
// coop_qr_scratch_bytes(grid) bytes, barrier state zero-initialised once, err is a
// device status word (kErrBarrierTimeout on a barrier that gave up).
struct GridBarrier;
size_t coop_qr_scratch_bytes(int max_grid);
int coop_qr_grid(long long m, int num_sms);
// co-resident CTAs of the cooperative QR on the current device (in *out)
cudaError_t coop_qr_max_grid(int* out);
cudaError_t householder_qr_coop(double2* M, long long m, int n, double2* R, int Rt, double2* tau_ws, double* scratch,
                                GridBarrier* bar, int* err, int grid, cudaStream_t s);
// Panel-blocked cooperative Householder QR (ttn_qr.cu), same conventions and arguments
// as householder_qr_coop but n <= kMaxBond; scratch of qr_blocked_scratch_bytes(grid)
// bytes; qr_blocked_max_grid() must run once before the first launch (it sets the
// kernels' shared-memory limit).
size_t qr_blocked_scratch_bytes(int max_grid);
int qr_blocked_max_grid();
cudaError_t householder_qr_blocked(double2* M, long long m, int n, double2* R, int Rt, double2* tau_ws,
                                   double* scratch, GridBarrier* bar, int* err, int grid, cudaStream_t s);
// Householder QR with every CTA's rows held in shared memory (ttn_qr_rows.cu), same
// conventions and arguments as householder_qr_blocked, n <= kMaxBond; at most
// qr_rows_max_rows(n) <= kQrRowsMax rows per CTA (else cudaErrorInvalidValue); scratch of
// qr_rows_scratch_bytes(grid) bytes; qr_rows_max_grid() must run once before the first
// launch (it sets the kernels' shared-memory limit).
constexpr int kQrRowsMax = 64;
size_t qr_rows_scratch_bytes(int max_grid);
int qr_rows_max_rows(int n);
int qr_rows_max_grid();
// phase (optional): 16 ns counters, see ttn_qr_rows.cu
constexpr int kQrPhases = 16;
cudaError_t householder_qr_rows(double2* M, long long m, int n, double2* R, int Rt, double2* tau_ws, double* scratch,
                                GridBarrier* bar, int* err, int grid, cudaStream_t s,
                                unsigned long long* phase = nullptr);
// r2l matricisation: M(y*pre + x, i) = A((x*dm + i)*post + y) and its inverse.
void permute_mode_last(const double2* A, double2* M, long long pre, int dm, long long post, cudaStream_t s);
void unpermute_mode_last(const double2* M, double2* A, long long pre, int dm, long long post, cudaStream_t s);

// ---- small helpers ------------------------------------------------------------------
void zcopy(double2* dst, const double2* src, long long n, cudaStream_t s);
// out = s*x (+ out when acc)
void zaxpy(double2* out, const double2* x, double2 s, long long n, bool acc, cudaStream_t st);
void zfill(double2* dst, double2 v, long long n, cudaStream_t s);
void zscale_identity(double2* dst, int r, double2 v, cudaStream_t s);
// out = sum_k diag(M)... trace of an r x r matrix into a device double2
void ztrace(const double2* M, int r, double2* out, cudaStream_t s);
// status word: set to code if any element is non-finite
void check_finite(const double2* x, long long n, int* status, int code, cudaStream_t s);

// FP64 FMA throughput of the current device (TFLOP/s), from a long FMA-chain kernel.
double measure_fp64_fma_tflops();

}  // namespace ttn
