// Persistent cooperative Krylov exponential: one launch evolves one node tensor (or
// bond matrix) by exp(coeff * tau * H), running every Lanczos iteration, the Expokit
// step control (Sidje, ACM TOMS 24, 1998) and every sub-step on the device.
//
// The matrix-vector product is a per-node program of contractions (mode products,
// mean-field products, axpys) compiled on the host from the term plan; the grid
// executes it phase by phase with grid barriers only where one contraction reads what
// another wrote.  Arithmetic per element matches the multi-kernel path.
#include "ttn_expm.cuh"
#include "ttn_coop.cuh"
#include "ttn_kernels.cuh"
#include "ttn_tc_core.cuh"

#include <cmath>

namespace ttn {

namespace {
constexpr int ET = 256;   // threads per CTA
constexpr int EQ = 72;    // max Krylov vectors

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ double2 cscale(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sums of q complex values per thread-slot; result in red2[0..nq)
struct Red {
  double2 w[ET / 32][EQ];
};

__device__ double2* buf_of(const ExpmArgs& a, int id, const double2* x) {
  switch (id) {
    case 0: return (double2*)x;
    case 1: return a.p;
    case 2: return a.t1;
    case 3: return a.t2;
    default: return a.t3;
  }
}

// one contraction of the matvec program over all output elements (grid-stride)
__device__ void run_op(const ExpmArgs& a, const MvOp& op, const double2* x) {
  const double2* in = buf_of(a, op.in, x);
  double2* out = buf_of(a, op.out, x);
  const long long nthreads = (long long)gridDim.x * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool acc = (op.beta != 0);
  if (op.kind == MV_MODE) {
    const int d = op.d;
    const long long nb = op.nb, total = op.na * d * nb;
    for (long long e = tid; e < total; e += nthreads) {
      const long long aa = e / (d * nb), rem = e % (d * nb);
      const int i = (int)(rem / nb);
      const long long b = rem % nb;
      const double2* S = op.mat + (long long)i * d;
      const double2* v = in + aa * d * nb + b;
      double2 s = make_double2(0.0, 0.0);
      for (int j = 0; j < d; ++j) s = cfma(S[j], v[(long long)j * nb], s);
      double2 r = cmul(op.alpha, s);
      if (acc) r = cadd(r, out[e]);
      out[e] = r;
    }
  } else if (op.kind == MV_MF) {
    const int r = op.d;
    const long long total = op.na * r;
    for (long long e = tid; e < total; e += nthreads) {
      const long long xx = e / r;
      const int k = (int)(e % r);
      const double2* v = in + xx * r;
      const double2* M = op.mat + (long long)k * r;
      double2 s = make_double2(0.0, 0.0);
      for (int l = 0; l < r; ++l) s = cfma(v[l], M[l], s);
      double2 o = cmul(op.alpha, s);
      if (acc) o = cadd(o, out[e]);
      out[e] = o;
    }
  } else if (op.kind == MV_AXPY) {
    const long long total = op.na;
    for (long long e = tid; e < total; e += nthreads) {
      double2 o = cmul(op.alpha, in[e]);
      if (acc) o = cadd(o, out[e]);
      out[e] = o;
    }
  } else {  // MV_ZERO
    for (long long e = tid; e < op.na; e += nthreads) out[e] = make_double2(0.0, 0.0);
  }
}

// ---- tensor-core contractions (mixed precision).  Per tile D(128 x 64) = A(128 x 128) B(64 x 128)^T
// in split TF32 with two FP32 accumulators in TMEM (hi*hi and hi*lo + lo*hi).
struct TcState {
  uint32_t tmem;      // TMEM base (128 columns)
  uint32_t phase;     // mbarrier parity
  uint64_t* mbar;
  uint32_t* a_hi;     // 128 x 128 tf32
  uint32_t* a_lo;
  uint32_t* b_hi;     // 64 x 128 tf32
  uint32_t* b_lo;
};
constexpr int TC_A_WORDS = 128 * 128, TC_B_WORDS = 64 * 128;
constexpr size_t TC_SMEM = (size_t)(2 * TC_A_WORDS + 2 * TC_B_WORDS) * 4;

__device__ __forceinline__ void put_a(TcState& t, int row, int k, double v) {
  uint32_t h, l;
  tc::split_tf32(v, h, l);
  const uint32_t o = tc::tf32_offset(row, k, 128) / 4;
  t.a_hi[o] = h;
  t.a_lo[o] = l;
}
__device__ __forceinline__ void put_b(TcState& t, int row, int k, double v) {
  uint32_t h, l;
  tc::split_tf32(v, h, l);
  const uint32_t o = tc::tf32_offset(row, k, 64) / 4;
  t.b_hi[o] = h;
  t.b_lo[o] = l;
}

// issue the 48 MMAs of one tile, wait for them; returns false on a timed-out wait
__device__ bool tc_tile_mma(TcState& t) {
  tc::fence_proxy_async();
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  if (threadIdx.x == 0) {
    const uint32_t idesc = tc::idesc_tf32(128, 64);
    const uint32_t lboA = 16 * 128, lboB = 8 * 128, sbo = 128;
    for (int kk = 0; kk < 16; ++kk) {
      const uint32_t offA = (uint32_t)kk * 2 * 16 * 128, offB = (uint32_t)kk * 2 * 8 * 128;
      const uint64_t ah = tc::smem_desc(tc::smem_u32(t.a_hi) + offA, lboA, sbo);
      const uint64_t al = tc::smem_desc(tc::smem_u32(t.a_lo) + offA, lboA, sbo);
      const uint64_t bh = tc::smem_desc(tc::smem_u32(t.b_hi) + offB, lboB, sbo);
      const uint64_t bl = tc::smem_desc(tc::smem_u32(t.b_lo) + offB, lboB, sbo);
      tc::mma_tf32(t.tmem, ah, bh, idesc, kk > 0);
      tc::mma_tf32(t.tmem + 64, ah, bl, idesc, kk > 0);
      tc::mma_tf32(t.tmem + 64, al, bh, idesc, 1);
    }
    tc::mma_commit(t.mbar);
  }
  __syncwarp();
  const bool ok = tc::mbar_wait(t.mbar, t.phase);
  t.phase ^= 1u;
  tc::fence_after();
  return ok;
}

// this thread's row (warps 0-3: rows 0..127) of the tile result, 16 columns starting at c0
__device__ __forceinline__ void tc_tile_row16(const TcState& t, int c0, double* v) {
  const int warp = threadIdx.x >> 5;
  float mv[16], cv[16];
  tc::tmem_ld16(t.tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, mv);
  tc::tmem_ld16(t.tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(64 + c0), cv);
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = (double)mv[i] + (double)cv[i];
}

__device__ void run_op_tc(const ExpmArgs& a, const MvOp& op, const double2* x, TcState& t) {
  const double2* in = buf_of(a, op.in, x);
  double2* out = buf_of(a, op.out, x);
  const int warp = threadIdx.x >> 5;
  const bool acc = (op.beta != 0);
  if (op.kind == MV_MODE) {
    // out(aa, i, b) = sum_j (alpha S)(i, j) in(aa, j, b); tiles of 64 columns b
    const long long nb = op.nb, tiles = op.na * (nb / 64);
    if ((long long)blockIdx.x >= tiles) return;
    // A = real block form of alpha*S, loaded once per op by every CTA that has a tile
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
      const int i = e / 64, j = e % 64;
      const double2 sv = cmul(op.alpha, op.mat[e]);
      put_a(t, i, j, sv.x);
      put_a(t, i, 64 + j, -sv.y);
      put_a(t, 64 + i, j, sv.y);
      put_a(t, 64 + i, 64 + j, sv.x);
    }
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
      const long long aa = tile / (nb / 64), b0 = (tile % (nb / 64)) * 64;
      const double2* src = in + aa * 64 * nb + b0;
      for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
        const int j = e / 64, n = e % 64;  // consecutive threads read consecutive b
        const double2 v = src[(long long)j * nb + n];
        put_b(t, n, j, v.x);
        put_b(t, n, 64 + j, v.y);
      }
      if (!tc_tile_mma(t) && threadIdx.x == 0) atomicOr(a.err, tc::kErrMmaTimeout);
      if (warp < 4) {
        const int row = threadIdx.x;  // 0..127: rows < 64 real parts, >= 64 imaginary parts
        const int i = row & 63;
        double* dst = (double*)(out + aa * 64 * nb + (long long)i * nb + b0) + (row >> 6);
        for (int c0 = 0; c0 < 64; c0 += 16) {
          double v[16];
          tc_tile_row16(t, c0, v);
#pragma unroll
          for (int n = 0; n < 16; ++n) dst[2 * (c0 + n)] = acc ? dst[2 * (c0 + n)] + v[n] : v[n];
        }
      }
      tc::fence_before();
      __syncthreads();
    }
  } else {
    // MF: out(x, k) = sum_l in(x, l) (alpha M)(k, l); tiles of 128 rows x, two column halves
    const long long nx = op.na, tiles = (nx / 128) * 2;
    if ((long long)blockIdx.x >= tiles) return;
    int loaded_half = -1;
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
      const long long xb = tile / 2;
      const int half = (int)(tile % 2);
      if (half != loaded_half) {
        for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
          const int k = e / 64, l = e % 64;
          const double2 mv = cmul(op.alpha, op.mat[e]);
          if (half == 0) {
            put_b(t, k, l, mv.x);
            put_b(t, k, 64 + l, -mv.y);
          } else {
            put_b(t, k, l, mv.y);
            put_b(t, k, 64 + l, mv.x);
          }
        }
        loaded_half = half;
      }
      const double2* src = in + xb * 128 * 64;
      for (int e = threadIdx.x; e < 128 * 64; e += blockDim.x) {
        const int r = e / 64, l = e % 64;
        const double2 v = src[e];
        put_a(t, r, l, v.x);
        put_a(t, r, 64 + l, v.y);
      }
      if (!tc_tile_mma(t) && threadIdx.x == 0) atomicOr(a.err, tc::kErrMmaTimeout);
      if (warp < 4) {
        const int row = threadIdx.x;
        double* dst = (double*)(out + (xb * 128 + row) * 64) + half;
        for (int c0 = 0; c0 < 64; c0 += 16) {
          double v[16];
          tc_tile_row16(t, c0, v);
#pragma unroll
          for (int k = 0; k < 16; ++k) dst[2 * (c0 + k)] = acc ? dst[2 * (c0 + k)] + v[k] : v[k];
        }
      }
      tc::fence_before();
      __syncthreads();
    }
  }
}

__device__ void run_program(const ExpmArgs& a, const double2* x, TcState* t) {
  for (int k = 0; k < a.nops; ++k) {
    const MvOp& op = a.prog[k];
    if (op.barrier_before) grid_barrier(a.bar, a.err);
    if (op.tc && t) run_op_tc(a, op, x, *t);
    else run_op(a, op, x);
  }
}

// ---- reductions: partials [gridDim][nq] (complex), reduced by every CTA in block order
__device__ void store_partials(Red& sm, int nq, double2* part) {
  __syncthreads();
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int w = 0; w < ET / 32; ++w) s = cadd(s, sm.w[w][q]);
    part[(long long)blockIdx.x * nq + q] = s;
  }
  __syncthreads();
}
// every CTA: out[q] = sum_b part[b][q], threads over (q, b-slices)
__device__ void reduce_partials(const double2* part, int nq, double2* out, Red& sm) {
  const int G = gridDim.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // warp w handles q = w, w+8, ...; lanes stride over b
  for (int q = w; q < nq; q += ET / 32) {
    double2 s = make_double2(0.0, 0.0);
    for (int b = lane; b < G; b += 32) s = cadd(s, part[(long long)b * nq + q]);
    s.x = wsum(s.x);
    s.y = wsum(s.y);
    if (lane == 0) out[q] = s;
  }
  __syncthreads();
}

__device__ double2 cexp_d(double2 x) {
  double ex = exp(x.x), sn, cs;
  sincos(x.y, &sn, &cs);
  return make_double2(ex * cs, ex * sn);
}
__device__ double cabs_d(double2 x) { return hypot(x.x, x.y); }
__device__ double2 cdiv_s(double2 a, double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  }
  double r = b.x / b.y, den = b.x * r + b.y;
  return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}
__device__ double2 phi1(double2 x) {
  if (cabs_d(x) < 0.5) {
    double2 s = make_double2(0.0, 0.0), t = make_double2(1.0, 0.0);
    for (int k = 1; k <= 18; ++k) {
      s = cadd(s, t);
      t = cscale(1.0 / double(k + 1), cmul(t, x));
    }
    return s;
  }
  double2 ex = cexp_d(x);
  return cdiv_s(make_double2(ex.x - 1.0, ex.y), x);
}
__device__ double2 phi2(double2 x) {
  if (cabs_d(x) < 0.5) {
    double2 s = make_double2(0.0, 0.0), t = make_double2(0.5, 0.0);
    for (int k = 2; k <= 20; ++k) {
      s = cadd(s, t);
      t = cscale(1.0 / double(k + 1), cmul(t, x));
    }
    return s;
  }
  double2 ex = cexp_d(x);
  return cdiv_s(make_double2(ex.x - 1.0 - x.x, ex.y - x.y), cmul(x, x));
}

// Implicit-QL eigen-decomposition (EISPACK tql2 scheme) by one warp: lane 0 runs the
// scalar recurrences and records the plane rotations, all lanes apply them to their
// rows of the eigenvector matrix.  Per element the operations are those of the
// sequential routine, in the same order.
struct CtlSmem {
  double z[64 * 64];
  double d[64], e[64];
  double rs[64], rc[64];
  int rot_lo, rot_hi, status;
  double2 F[66];
};

__device__ int warp_tql2(int n, CtlSmem& S) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < n * n; i += 32) S.z[i] = ((i / n) == (i % n)) ? 1.0 : 0.0;
  __syncwarp();
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      if (lane == 0) {
        int m;
        double* d = S.d;
        double* e = S.e;
        for (m = l; m < n - 1; ++m) {
          double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= 1e-300 + 2.220446049250313e-16 * dd) break;
        }
        S.status = 0;
        S.rot_lo = S.rot_hi = 0;
        if (m == l) {
          S.status = 1;  // converged
        } else if (++iter > 60) {
          S.status = 2;  // failed
        } else {
          double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
          double r = hypot(g, 1.0);
          g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? fabs(r) : -fabs(r)));
          double s = 1.0, c = 1.0, p = 0.0;
          int i;
          bool underflow = false;
          S.rot_hi = m - 1;
          for (i = m - 1; i >= l; --i) {
            double f = s * e[i], b = c * e[i];
            r = hypot(f, g);
            e[i + 1] = r;
            if (r == 0.0) {
              d[i + 1] -= p;
              e[m] = 0.0;
              underflow = true;
              break;
            }
            s = f / r;
            c = g / r;
            g = d[i + 1] - p;
            r = (d[i] - g) * s + 2.0 * c * b;
            p = s * r;
            d[i + 1] = g + p;
            g = c * r - b;
            S.rs[i] = s;
            S.rc[i] = c;
          }
          S.rot_lo = underflow ? i + 1 : l;
          if (!underflow) {
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
          }
          S.status = underflow ? 3 : 0;
        }
      }
      __syncwarp();
      const int st = S.status;
      if (st == 1) break;
      if (st == 2) return 1;
      // apply the recorded rotations i = rot_hi .. rot_lo to every row k (lane-parallel)
      const int hi = S.rot_hi, lo = S.rot_lo;
      for (int k = lane; k < n; k += 32) {
        for (int i = hi; i >= lo; --i) {
          double s = S.rs[i], c = S.rc[i];
          double f = S.z[k * n + i + 1];
          S.z[k * n + i + 1] = s * S.z[k * n + i] + c * f;
          S.z[k * n + i] = c * S.z[k * n + i] - s * f;
        }
      }
      __syncwarp();
    }
  }
  return 0;
}

// Expokit step control by warp 0 of block 0.
__device__ void control(const ExpmArgs& a, CtlSmem& S) {
  KrylovCtl* ctl = a.ctl;
  const int lane = threadIdx.x & 31;
  if (ctl->done) {
    for (int q = lane; q < 2 * 72; q += 32) ctl->coef[q] = 0.0;
    return;
  }
  const int m = ctl->m, mb = ctl->mb, k1 = ctl->k1;
  const double tol = ctl->tol, gamma = 0.9, delta = 1.2;
  const double beta = ctl->beta, avnorm = ctl->avnorm;
  for (int i = lane; i < mb; i += 32) {
    S.d[i] = ctl->alpha[i];
    S.e[i] = (i + 1 < mb) ? ctl->bet[i + 1] : 0.0;
  }
  __syncwarp();
  if (warp_tql2(mb, S)) {
    if (lane == 0) {
      ctl->err |= 4;
      ctl->done = 1;
    }
    return;
  }
  __shared__ double s_tstep, s_err, s_xm;
  __shared__ int s_accept, s_fail;
  if (lane == 0) {
    double t_step = fmin(ctl->t_out - ctl->t_now, ctl->t_new);
    if (k1 == 0) t_step = ctl->t_out - ctl->t_now;
    s_tstep = t_step;
    s_fail = 0;
  }
  __syncwarp();
  const double2 cf = make_double2(ctl->cf_re, ctl->cf_im);
  int ireject = 0;
  for (;;) {
    const double t_step = s_tstep;
    const double2 zc = cscale(ctl->sgn * t_step, cf);
    for (int i = lane; i < mb; i += 32) {
      double2 s = make_double2(0.0, 0.0);
      for (int q = 0; q < mb; ++q) {
        double2 ex = cexp_d(cscale(S.d[q], zc));
        s = cadd(s, cscale(S.z[i * mb + q] * S.z[q], ex));
      }
      S.F[i] = s;
    }
    __syncwarp();
    if (lane == 0) {
      double err_loc, xm = 1.0 / m;
      int accept = 0;
      if (k1 == 0) {
        err_loc = 1e-14;
        accept = 1;
      } else {
        double2 f1 = make_double2(0.0, 0.0), f2 = make_double2(0.0, 0.0);
        for (int q = 0; q < mb; ++q) {
          double2 x = cscale(S.d[q], zc);
          double w = S.z[(mb - 1) * mb + q] * S.z[q];
          f1 = cadd(f1, cscale(w, cmul(zc, phi1(x))));
          f2 = cadd(f2, cscale(w, cmul(cmul(zc, zc), phi2(x))));
        }
        S.F[mb] = cscale(ctl->bet[mb], f1);
        S.F[mb + 1] = cscale(ctl->bet[mb], f2);
        double p1 = cabs_d(S.F[mb]) * beta, p2 = cabs_d(S.F[mb + 1]) * beta * avnorm;
        if (p1 > 10.0 * p2) {
          err_loc = p2;
          xm = 1.0 / m;
        } else if (p1 > p2) {
          err_loc = p1 * p2 / (p1 - p2);
          xm = 1.0 / m;
        } else {
          err_loc = p1;
          xm = 1.0 / (m - 1);
        }
        if (err_loc <= delta * t_step * tol) accept = 1;
      }
      s_err = err_loc;
      s_xm = xm;
      s_accept = accept;
      if (!accept) {
        if (ireject == 10) {
          s_fail = 1;
        } else {
          double ts = gamma * t_step * pow(t_step * tol / err_loc, xm);
          double sc = pow(10.0, floor(log10(ts)) - 1.0);
          s_tstep = ceil(ts / sc) * sc;
        }
      }
    }
    __syncwarp();
    if (s_accept || s_fail) break;
    ++ireject;
  }
  if (lane == 0) {
    const double t_step = s_tstep, err_loc = s_err, xm = s_xm;
    if (s_fail) {
      ctl->err |= 1;
      ctl->done = 1;
    } else if (!isfinite(t_step) || !(t_step > 0.0) || !isfinite(err_loc)) {
      ctl->err |= 8;
      ctl->done = 1;
    } else {
      const int mx = mb + (k1 > 1 ? k1 - 1 : 0);
      for (int q = 0; q < 72; ++q) {
        double2 c = (q < mx) ? cscale(beta, S.F[q]) : make_double2(0.0, 0.0);
        ctl->coef[2 * q] = c.x;
        ctl->coef[2 * q + 1] = c.y;
      }
      ctl->t_now += t_step;
      if (k1 != 0) {
        double tn = gamma * t_step * pow(t_step * tol / fmax(err_loc, 1e-300), xm);
        double sc = pow(10.0, floor(log10(tn)) - 1.0);
        ctl->t_new = ceil(tn / sc) * sc;
        if (!isfinite(ctl->t_new) || !(ctl->t_new > 0.0)) ctl->t_new = t_step;
      }
      ctl->napps += mb + (k1 != 0 ? 1 : 0);
      ctl->substeps += 1;
      if (ctl->t_now >= ctl->t_out) ctl->done = 1;
    }
  }
  __syncwarp();
}

__global__ void __launch_bounds__(ET, 2) k_expm_coop(ExpmArgs a) {
  __shared__ Red sm;
  __shared__ double2 red[EQ];
  __shared__ int s_done;
  __shared__ __align__(8) uint64_t s_mbar;
  __shared__ uint32_t s_tmem;
  extern __shared__ __align__(1024) unsigned char dsm[];
  // the controller's scratch and the tensor-core operands share the dynamic buffer: they
  // are used in different phases
  CtlSmem& cs = *reinterpret_cast<CtlSmem*>(dsm);
  TcState tcs;
  TcState* tcp = nullptr;
  if (a.mixed) {
    if (threadIdx.x == 0) tc::mbar_init(&s_mbar, 1);
    if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&s_tmem, 128);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    tcs.tmem = s_tmem;
    tcs.phase = 0;
    tcs.mbar = &s_mbar;
    tcs.a_hi = reinterpret_cast<uint32_t*>(dsm);
    tcs.a_lo = tcs.a_hi + TC_A_WORDS;
    tcs.b_hi = tcs.a_lo + TC_A_WORDS;
    tcs.b_lo = tcs.b_hi + TC_B_WORDS;
    tcp = &tcs;
  }
  KrylovCtl* ctl = a.ctl;
  const long long n = a.n;
  const long long nthreads = (long long)gridDim.x * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int m = a.m;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double2* pa = a.part;
  double2* pb = a.part + (size_t)gridDim.x * EQ;

  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->m = m;
    ctl->t_out = fabs(a.tau);
    ctl->sgn = a.tau >= 0.0 ? 1.0 : -1.0;
    ctl->t_now = 0.0;
    ctl->t_new = fabs(a.tau);
    ctl->cf_re = a.cf_re;
    ctl->cf_im = a.cf_im;
    ctl->tol = a.tol;
    ctl->done = (a.tau == 0.0) ? 1 : 0;
    ctl->err = 0;
    ctl->substeps = 0;
    ctl->napps = 0;
    for (int q = 0; q < 73; ++q) ctl->bet[q] = 0.0;
  }
  if (a.apply_only) {
    grid_barrier(a.bar, a.err);
    run_program(a, a.y, tcp);
    grid_barrier(a.bar, a.err);
  }
  for (int sub = 0; sub < (a.apply_only ? 0 : 100000); ++sub) {
    grid_barrier(a.bar, a.err);
    if (threadIdx.x == 0) s_done = *(volatile int*)&ctl->done;
    __syncthreads();
    if (s_done) break;
    // ---- begin: beta = ||y||, V0 = y / beta
    {
      double s = 0.0;
      for (long long i = tid; i < n; i += nthreads) {
        double2 v = a.y[i];
        s += v.x * v.x + v.y * v.y;
      }
      s = wsum(s);
      if (lane == 0) sm.w[warp][0] = make_double2(s, 0.0);
      store_partials(sm, 1, pa);
    }
    grid_barrier(a.bar, a.err);
    reduce_partials(pa, 1, red, sm);
    {
      const double beta = sqrt(red[0].x);
      const double inv = beta > 0.0 ? 1.0 / beta : 0.0;
      for (long long i = tid; i < n; i += nthreads) a.V[i] = cscale(inv, a.y[i]);
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->beta = beta;
        ctl->mb = m;
        ctl->k1 = 2;
        if (!(beta > 0.0) || !isfinite(beta)) {
          ctl->done = 1;
          if (!isfinite(beta)) ctl->err |= 2;
        }
      }
    }
    // ---- Lanczos with full re-orthogonalisation
    for (int j = 0; j < m; ++j) {
      const double2* Vj = a.V + (long long)j * a.ldv;
      grid_barrier(a.bar, a.err);
      run_program(a, Vj, tcp);
      // partial <V_j, p> over my elements (same element ownership as the last writes of p)
      {
        double2 s = make_double2(0.0, 0.0);
        for (long long i = tid; i < n; i += nthreads) s = cadd(s, cmulc(Vj[i], a.p[i]));
        s.x = wsum(s.x);
        s.y = wsum(s.y);
        if (lane == 0) sm.w[warp][0] = s;
        store_partials(sm, 1, pa);
      }
      grid_barrier(a.bar, a.err);
      reduce_partials(pa, 1, red, sm);
      const double alpha = red[0].x;
      const double bj = (j > 0) ? ctl->bet[j] : 0.0;
      const double2* Vm = a.V + (long long)(j > 0 ? j - 1 : 0) * a.ldv;
      for (long long i = tid; i < n; i += nthreads) {
        double2 x = a.p[i], vj = Vj[i];
        x.x -= alpha * vj.x;
        x.y -= alpha * vj.y;
        if (j > 0) {
          double2 vm = Vm[i];
          x.x -= bj * vm.x;
          x.y -= bj * vm.y;
        }
        a.p[i] = x;
      }
      for (int q = 0; q <= j; ++q) {
        const double2* Vq = a.V + (long long)q * a.ldv;
        double2 s = make_double2(0.0, 0.0);
        for (long long i = tid; i < n; i += nthreads) s = cadd(s, cmulc(Vq[i], a.p[i]));
        s.x = wsum(s.x);
        s.y = wsum(s.y);
        if (lane == 0) sm.w[warp][q] = s;
      }
      store_partials(sm, j + 1, pb);
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->alpha[j] = alpha;
      grid_barrier(a.bar, a.err);
      reduce_partials(pb, j + 1, red, sm);
      {
        double s = 0.0;
        for (long long i = tid; i < n; i += nthreads) {
          double2 x = a.p[i];
          for (int q = 0; q <= j; ++q) x = csub(x, cmul(red[q], a.V[(long long)q * a.ldv + i]));
          a.p[i] = x;
          s += x.x * x.x + x.y * x.y;
        }
        s = wsum(s);
        if (lane == 0) sm.w[warp][0] = make_double2(s, 0.0);
        store_partials(sm, 1, pa);
      }
      grid_barrier(a.bar, a.err);
      reduce_partials(pa, 1, red, sm);
      {
        const double beta = sqrt(red[0].x);
        double anorm = 0.0;
        for (int q = 0; q <= j; ++q) {
          double nb = (q < j) ? ctl->bet[q + 1] : beta;
          double v = fabs(ctl->alpha[q]) + ctl->bet[q] + nb;
          anorm = v > anorm ? v : anorm;
        }
        const int brk = (beta <= 1e-14 * (1.0 + anorm)) ? 1 : 0;
        const double inv = brk ? 0.0 : 1.0 / beta;
        double2* Vn = a.V + (long long)(j + 1) * a.ldv;
        for (long long i = tid; i < n; i += nthreads) Vn[i] = cscale(inv, a.p[i]);
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          ctl->bet[j + 1] = brk ? 0.0 : beta;
          if (brk && ctl->mb == m) {
            ctl->mb = j + 1;
            ctl->k1 = 0;
          }
          if (!isfinite(beta)) ctl->err |= 2;
        }
        __syncthreads();
      }
    }
    // ---- ||H V_m|| for the error estimate
    grid_barrier(a.bar, a.err);
    run_program(a, a.V + (long long)m * a.ldv, tcp);
    {
      double s = 0.0;
      for (long long i = tid; i < n; i += nthreads) {
        double2 v = a.p[i];
        s += v.x * v.x + v.y * v.y;
      }
      s = wsum(s);
      if (lane == 0) sm.w[warp][0] = make_double2(s, 0.0);
      store_partials(sm, 1, pa);
    }
    grid_barrier(a.bar, a.err);
    if (blockIdx.x == 0) {
      reduce_partials(pa, 1, red, sm);
      if (threadIdx.x == 0) ctl->avnorm = sqrt(red[0].x);
      __syncthreads();
      if (warp == 0) control(a, cs);
    }
    grid_barrier(a.bar, a.err);
    // ---- y = sum_q c_q V_q
    {
      for (int q = threadIdx.x; q <= m; q += blockDim.x)
        red[q] = make_double2(ctl->coef[2 * q], ctl->coef[2 * q + 1]);
      __syncthreads();
      for (long long i = tid; i < n; i += nthreads) {
        double2 s = make_double2(0.0, 0.0);
        for (int q = 0; q <= m; ++q) s = cfma(red[q], a.V[(long long)q * a.ldv + i], s);
        a.y[i] = s;
      }
      __syncthreads();
    }
  }
  if (a.mixed) {
    tc::fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
      tc::fence_after();
      tc::tmem_dealloc(tcs.tmem, 128);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && !a.apply_only) {
    if (a.napps_total) atomicAdd((unsigned long long*)a.napps_total, (unsigned long long)ctl->napps);
    if (a.flops_total) atomicAdd(a.flops_total, a.flops_per_app * (double)ctl->napps);
    int e = ctl->err;
    if (!ctl->done) e |= 16;  // sub-step limit reached
    if (e) atomicOr(a.err, e << kKrylovErrShift);
  }
}
}  // namespace

static size_t dyn_smem(int mixed) { return mixed ? (TC_SMEM > sizeof(CtlSmem) ? TC_SMEM : sizeof(CtlSmem)) : sizeof(CtlSmem); }

int expm_coop_max_grid(int mixed) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(k_expm_coop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem(1));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_expm_coop, ET, dyn_smem(mixed));
  return sms * (per < 1 ? 1 : per);
}

size_t expm_partial_bytes(int max_grid) { return (size_t)2 * max_grid * EQ * sizeof(double2); }

cudaError_t expm_coop(const ExpmArgs& a, int grid, cudaStream_t s) {
  ExpmArgs b = a;
  void* args[] = {&b};
  ++g_launches;
  return cudaLaunchCooperativeKernel((const void*)k_expm_coop, dim3(grid), dim3(ET), args, dyn_smem(a.mixed), s);
}

}  // namespace ttn
