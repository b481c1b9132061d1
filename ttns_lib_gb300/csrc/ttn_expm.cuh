// Persistent cooperative Krylov exponential (see ttn_expm.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "ttn_kernels.cuh"

namespace ttn {

struct GridBarrier;

enum { MV_MODE = 0, MV_MF = 1, MV_AXPY = 2, MV_ZERO = 3, MV_CSR = 4 };

// One contraction of a matrix-vector program.  Buffers: 0 = input vector, 1 = output,
// 2..4 = temporaries.  MODE: out(a,i,b) = alpha sum_j mat(i,j) in(a,j,b) (+ out) with
// shape (na, d, nb); MF: out(x,k) = alpha sum_l in(x,l) mat(k,l) (+ out) with nx = na,
// r = d; AXPY: out = alpha in (+ out) over na elements; ZERO: out = 0 over na elements;
// CSR: MODE with a sparse d x d matrix (row i: mat[q], column colind[q] for q in
// rowptr[i] .. rowptr[i+1]), for sparse leaf operators.
struct MvOp {
  int kind;
  int in, out;
  int barrier_before;
  const double2* mat;
  long long na, nb;
  int d;
  int beta;  // 1: accumulate into out
  int tc;    // 1: run on the tensor cores (mixed precision; MODE with d = 64, MF with r = 64)
  int img;   // tensor-core ops: slot of the operator image (split TF32 block form of alpha mat)
  double2 alpha;
  const int* rowptr;  // CSR only
  const int* colind;
};
// bytes of one operator image: row exponents (1 KB) and the 128 x 128 block operand as
// six bf16 integer slices in four K-chunks of 48 KB
constexpr size_t kTcImageBytes = (size_t)1024 + (size_t)4 * 6 * 128 * 32 * 2;

struct ExpmArgs {
  double2* y;            // vector evolved in place
  long long n;
  double2* V;            // Krylov basis, m+1 vectors, stride ldv
  long long ldv;
  double2 *p, *t1, *t2, *t3;
  const MvOp* prog;      // device program
  int nops;
  double2* part;         // reduction partials (expm_partial_bytes)
  KrylovCtl* ctl;
  GridBarrier* bar;
  int* err;              // status word (Krylov error bits, barrier timeout)
  long long* napps_total;  // device counter of H applications (may be null)
  double* flops_total;     // device counter of algorithmic matvec flops (may be null)
  double flops_per_app;    // flops of one application of the program
  int m;
  double tau, cf_re, cf_im, tol;
  int mixed;             // 1: the program contains tensor-core contractions (TMEM + big smem)
  int apply_only;        // 1: apply the program once to y (result in p) and return
  int krylov_stop;       // 1: end a sub-step's Lanczos recurrence once the residual estimate
                         //    for the remaining interval is below tol (FP64 programs only)
  unsigned long long* phase;  // optional: ns spent per phase as seen by CTA 0 (kPhases slots)
  uint32_t* tc_img;      // operator images of the tensor-core ops (kTcImageBytes each)
  MvOp op1;              // the program when prog is null (one contraction, apply_only)
  int tail_barrier;      // 1: a grid barrier after the program (tensor-core writes to p
                         // are distributed by tiles, not by the element-wise ownership the
                         // Lanczos passes assume)
  int tpo;               // lanes per output element of the element-wise program ops (1, 2, 4
                         // or 8; above 1 the program needs tail_barrier)
  int smem_vecs;         // 1 (one-CTA launches of small problems): the basis V, p and the
                         // temporaries live in the launch's shared memory, ldt elements
                         // each, instead of at V / p / t1..t3
  long long ldt;
};
constexpr int kPhases = 16;  // begin, matvec, alpha, reorth coefficients, reorth + norm,
                             // ||H V_m||, control, combine, sub-steps, launches; then inside
                             // the tensor-core contractions: row exponents, chunk pipeline,
                             // TMEM drain, output, tiles

// co-resident CTAs for the plain (mixed = 0) or tensor-core (mixed = 1) configuration
int expm_coop_max_grid(int mixed);
size_t expm_partial_bytes(int max_grid);
// threads per CTA: a multiple of 32 up to 256 (tensor-core programs always use 256)
cudaError_t expm_coop(const ExpmArgs& a, int grid, cudaStream_t s, int threads = 256);
// shared memory of a one-CTA launch with the vectors resident (smem_vecs): m + 5 vectors of
// ldt elements after the controller's scratch; and the most a launch may take
size_t expm_smem_vecs_bytes(int m, long long ldt);
size_t expm_smem_vecs_max_bytes();
// whether a contraction can run on the tensor cores
// Tensor-core contractions need rank-64 operands and enough 64-column tiles to occupy the
// device; smaller ones run faster as element-wise FP64 contractions.
// A tile is the 64 outputs of the operator times kTcTileN columns of the input.
constexpr int kTcTileN = 32;
constexpr long long kTcMinTiles = 64;
inline bool tc_eligible(int kind, int d, long long na, long long nb) {
  if (kind == MV_MODE) return d == 64 && nb % kTcTileN == 0 && na * (nb / kTcTileN) >= kTcMinTiles;
  if (kind == MV_MF) return d == 64 && na % kTcTileN == 0 && na / kTcTileN >= kTcMinTiles;
  return false;
}

}  // namespace ttn
