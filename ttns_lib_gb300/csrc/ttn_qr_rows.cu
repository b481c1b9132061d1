// Cooperative Householder QR of a tall complex matrix (m x n, n <= 64, row-major, in
// place) with every CTA's rows resident in shared memory for the whole factorisation:
// M <- Q (m x n), R (n x n) upper triangular, LAPACK zgeqrf / zungqr conventions (zlarfg
// reflectors: real beta, tau = (beta - alpha) / beta, v(1) = 1, the safe-minimum rescaling
// of tiny columns; H^H = I - conj(tau) v v^H from the left; Q = H_0 ... H_{n-1} [I; 0]),
// the same algorithm as the panel-blocked kernel of ttn_qr.cu.
//
// Why a second kernel: on GB300 one SM issues a warp's FP64 instruction in 16 cycles and a
// dependent FP64 operation takes 64, so the panel-blocked kernel, whose 256 threads all
// repeat the scalar work of every column and which re-reads its rows from L2 after every
// grid barrier, spends each column waiting on its own FP64 pipe and on L2 (ncu: 35-41 %
// FP64 pipe, warps mostly stalled at block barriers; 15-22 us per column).  Here
//   * the rows live in shared memory (a stride of n | 1 complex keeps a warp's column
//     accesses free of bank conflicts) and are written back once at the end;
//   * per column, warp w alone forms slot w of the partials (w = 0: the column's squared
//     norm, w >= 1: its products with panel column j + w) and publishes it straight to
//     the scratch, so no block barrier precedes the grid barrier;
//   * the partials are summed without power-of-two rescaling while the CTA's column
//     maximum lies in [2^-400, 2^100] (squares and products then stay normal), the
//     rescaled form of ttn_qr.cu only otherwise;
//   * the reflector is formed by one thread, the update of the panel columns by one
//     thread per row, so no FP64 instruction is repeated by idle warps.
// The trailing columns are updated once per panel of 8 with the compact WY form (zlarft /
// zlarfb), whose V^H [V | M] partials are reduced cooperatively, and Q is formed backwards
// panel by panel (zungqr).  A CTA holds at most kQrRowsMax rows, fewer for wide matrices
// (qr_rows_max_rows: the rows and the per-CTA state share the opt-in shared memory).  Two
// instantiations: matrices of up to 64 columns, and of up to kMaxBond (bonds that subspace
// expansion grows past 64).
#include "ttn_coop.cuh"
#include "ttn_kernels.cuh"

#include <climits>
#include <cstdint>

namespace ttn {
namespace {

constexpr int QT = 256;                 // threads per CTA
constexpr int QW = QT / 32;             // warps
constexpr int QNB = 8;                  // panel width: one warp per panel column slot
// BN: widest matrix of an instantiation (64, or kMaxBond for the bonds that subspace
// expansion grows past 64); BN / QNB panels at most; QNB (QNB + BN) complex entries in one
// panel block V^H [V | M_trailing]
template <int BN> __host__ __device__ constexpr int qnp() { return BN / QNB; }
template <int BN> __host__ __device__ constexpr int qpw() { return QNB * (QNB + BN); }
constexpr int kNoScale = -100000;       // scale exponent published by a CTA with a zero column
constexpr int kQrPartsPerLane = 8;      // column partials per lane in the reduction: grids up to 256
static_assert(QW == QNB, "one warp per panel column slot");

struct RqrArgs {
  double2* M;
  long long m;
  int n;
  double2* R;
  int Rt;
  double2* tau_out;
  double* scr;
  GridBarrier* bar;
  int* err;
  unsigned long long* phase;  // optional: ns per phase as seen by thread 0 of CTA 0 (kQrPhases slots)
};

// wall time per phase as seen by thread 0 of CTA 0: column barrier, column sums, reflector,
// w, row update, next partials, panel updates (factorisation), R and Q formation; slot 8
// counts columns
struct QrClock {
  unsigned long long* acc;
  unsigned long long t;
  __device__ void mark(int k) {
    if (acc) {
      unsigned long long now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
      acc[k] += now - t;
      t = now;
    }
  }
};

// scratch layout (doubles), G = gridDim.x
//   colp [2][G][2 + 2 QNB]  per CTA, for the current column j: [0] its scale exponent e
//                           (0: unscaled, kNoScale: zero column), [1] sum |x 2^-e|^2 over
//                           its rows below the diagonal, [2w, 2w+1] sum conj(x 2^-e) M[:, j+w]
//   rowj [2][2 QNB]         M[j][j .. jend) from the CTA holding row j
//   pp   [G][2 qpw]         panel block partials;  pr [2 qpw] their sums
//   vt   [qnp][2 QNB QNB]   the top block of every panel's V (Q formation)
__host__ __device__ constexpr size_t rq_colw() { return 2 + 2 * QNB; }
__host__ __device__ constexpr size_t rq_off_rowj(int G) { return (size_t)2 * G * rq_colw(); }
__host__ __device__ constexpr size_t rq_off_pp(int G) { return rq_off_rowj(G) + 4 * QNB; }
template <int BN> __host__ __device__ constexpr size_t rq_off_pr(int G) { return rq_off_pp(G) + (size_t)2 * qpw<BN>() * G; }
template <int BN> __host__ __device__ constexpr size_t rq_off_vt(int G) { return rq_off_pr<BN>(G) + 2 * qpw<BN>(); }
template <int BN> __host__ __device__ constexpr size_t rq_doubles(int G) {
  return rq_off_vt<BN>(G) + (size_t)qnp<BN>() * 2 * QNB * QNB;
}

__device__ __forceinline__ double2 qadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 qmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 qmulc(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 qfms(double2 c, double2 a, double2 b) {  // c - a * b
  c.x = fma(-a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(-a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ double2 qfmac(double2 c, double2 a, double2 b) {  // c + conj(a) * b
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}
// floor(log2(x)) for finite x > 0 (subnormals included), from the bits
__device__ __forceinline__ int qilog2(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e != 0) return e - 1023;
  return -1074 + (63 - __clzll((long long)(b & 0xFFFFFFFFFFFFFull)));
}
// x * 2^k, exact while the result is normal; scalings below 2^-2000 give 0
__device__ __forceinline__ double qldexp(double x, int k) {
  if (k < -2000) return 0.0;
  if (k > 2000) k = 2000;
  if (k > 1000) {
    x *= __longlong_as_double((long long)(1000 + 1023) << 52);
    k -= 1000;
  } else if (k < -1000) {
    x *= __longlong_as_double((long long)(-1000 + 1023) << 52);
    k += 1000;
  }
  return x * __longlong_as_double((long long)(k + 1023) << 52);
}
__device__ __forceinline__ unsigned long long qabsmax_bits(double2 v) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long b = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
  return a > b ? a : b;
}
__device__ double qlapy3(double x, double y, double z) {
  double w = fmax(fabs(x), fmax(fabs(y), fabs(z)));
  if (w == 0.0) return 0.0;
  double a = x / w, b = y / w, c = z / w;
  return w * sqrt(a * a + b * b + c * c);
}
__device__ double2 qdiv(double2 a, double2 b) {  // Smith's division
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  }
  double r = b.x / b.y, den = b.x * r + b.y;
  return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

// per-CTA state, at the start of the dynamic shared memory (the rows follow it)
template <int BN>
struct RSmem {
  double2 tau[BN];
  double2 T[BN / QNB][QNB][QNB];  // compact WY factors of every panel
  double2 P[QNB][QNB + BN];       // reduced panel block (Gram | projections)
  double2 W[QNB][QNB + BN];       // T^H P (factorisation) or T P (Q formation)
  double2 g[QNB];               // Gram sums of column j with the panel columns, relative to 2^E
  double2 rowj[QNB];            // M[j][j .. jend), read next to the partials
  double2 w[QNB];               // conj(tau) conj(v)^T M[:, c] for the panel columns c
  double nrm2;                  // squared norm below the diagonal, relative to 2^(2E)
  int E;
  double2 scal, beta;
  int kx, kfac, active;
};

// the rows of this CTA in shared memory: row i (r0 <= i < r1) at rows[(i - r0) * lds]
struct Rows {
  double2* p;
  long long r0, r1;
  int lds;
  __device__ double2& at(long long i, int c) const { return p[(i - r0) * lds + c]; }
  // V(i, k) of the panel starting at column j0: 0 above the diagonal, 1 on it, M below
  __device__ double2 v(long long i, int j0, int k) const {
    const long long d = j0 + k;
    if (i < d) return make_double2(0.0, 0.0);
    if (i == d) return make_double2(1.0, 0.0);
    return at(i, (int)d);
  }
};

// Partials of column j (panel columns up to jend) over my rows, published by warp w for
// slot w; the row j entries by the CTA that holds row j.  A one-CTA launch writes the sums
// straight into S (what col_reduce would make of a single partial).
template <int BN>
__device__ void col_partials(const RqrArgs& a, const Rows& R, int j, int jend, RSmem<BN>& S) {
  const int G = gridDim.x, b = blockIdx.x, par = j & 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nc = jend - j - 1;
  double* cp = a.scr + ((size_t)par * G + b) * rq_colw();
  const long long lo = R.r0 > j + 1 ? R.r0 : j + 1;
  if (w <= nc) {
    unsigned long long um = 0;
    for (long long i = lo + lane; i < R.r1; i += 32) {
      const unsigned long long t = qabsmax_bits(R.at(i, j));
      um = t > um ? t : um;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, um, o);
      um = t > um ? t : um;
    }
    const double lmax = __longlong_as_double((long long)um);
    int e = 0;
    if (lmax > 0.0 && (lmax < 0x1p-400 || lmax > 0x1p100)) e = qilog2(lmax);
    double2 acc = make_double2(0.0, 0.0);
    for (long long i = lo + lane; i < R.r1; i += 32) {
      double2 x = R.at(i, j);
      if (e) {
        x.x = qldexp(x.x, -e);
        x.y = qldexp(x.y, -e);
      }
      if (w == 0) {
        acc.x = fma(x.x, x.x, acc.x);
        acc.x = fma(x.y, x.y, acc.x);
      } else {
        acc = qfmac(acc, x, R.at(i, j + w));
      }
    }
    if (w) {
      acc = warp_sum2(acc);
    } else {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    }
    if (lane == 0) {
      if (G == 1) {
        if (w == 0) {
          S.nrm2 = acc.x;
          S.E = lmax > 0.0 ? e : 0;
        } else {
          S.g[w] = acc;
        }
      } else if (w == 0) {
        reinterpret_cast<long long*>(cp)[0] = (long long)(lmax > 0.0 ? e : kNoScale);
        cp[1] = acc.x;
      } else {
        cp[2 * w] = acc.x;
        cp[2 * w + 1] = acc.y;
      }
    }
  }
  if (j >= R.r0 && j < R.r1 && w == QW - 1 && lane <= nc) {
    const double2 v = R.at(j, j + lane);
    if (G == 1) {
      S.rowj[lane] = v;
    } else {
      double* rj = a.scr + rq_off_rowj(G) + (size_t)par * 2 * QNB;
      rj[2 * lane] = v.x;
      rj[2 * lane + 1] = v.y;
    }
  }
}

// After the grid barrier: the column's sums over all CTAs (warp w: slot w) into S.
template <int BN>
__device__ void col_reduce(const RqrArgs& a, int j, int jend, RSmem<BN>& S) {
  const int G = gridDim.x, par = j & 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int nc = jend - j - 1;
  if (G == 1) return;  // col_partials wrote S
  // row j of the panel (alpha and the entries the w_c need), loaded by the last warp while
  // the others load the partials
  if (w == QW - 1 && lane <= nc) {
    const double* rj = a.scr + rq_off_rowj(G) + (size_t)par * 2 * QNB;
    S.rowj[lane] = make_double2(rj[2 * lane], rj[2 * lane + 1]);
  }
  if (w > nc) return;
  const double* cp = a.scr + (size_t)par * G * rq_colw();
  // every partial of this slot loaded at once (one L2 round trip), then the common scale
  long long ev[kQrPartsPerLane];
  double xv[kQrPartsPerLane], yv[kQrPartsPerLane];
#pragma unroll
  for (int u = 0; u < kQrPartsPerLane; ++u) {
    const int q = lane + 32 * u;
    ev[u] = kNoScale;
    xv[u] = yv[u] = 0.0;
    if (q < G) {
      const double* c = cp + (size_t)q * rq_colw();
      ev[u] = reinterpret_cast<const long long*>(c)[0];
      xv[u] = c[w == 0 ? 1 : 2 * w];
      if (w) yv[u] = c[2 * w + 1];
    }
  }
  int emax = kNoScale;
  bool scaled = false;
#pragma unroll
  for (int u = 0; u < kQrPartsPerLane; ++u) {
    const int e = (int)ev[u];
    emax = e > emax ? e : emax;
    scaled = scaled || (e != 0 && e != kNoScale);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const int t = __shfl_xor_sync(0xffffffffu, emax, o);
    emax = t > emax ? t : emax;
  }
  scaled = __any_sync(0xffffffffu, scaled);
  const int E = (emax == kNoScale) ? 0 : emax;
  double2 s = make_double2(0.0, 0.0);
#pragma unroll
  for (int u = 0; u < kQrPartsPerLane; ++u) {
    const int e = (int)ev[u];
    if (e == kNoScale) continue;
    if (w == 0) {
      s.x += scaled ? qldexp(xv[u], 2 * (e - E)) : xv[u];
    } else {
      s.x += scaled ? qldexp(xv[u], e - E) : xv[u];
      s.y += scaled ? qldexp(yv[u], e - E) : yv[u];
    }
  }
  if (w) {
    s = warp_sum2(s);
  } else {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
  }
  if (lane == 0) {
    if (w == 0) {
      S.nrm2 = s.x;
      S.E = E;
    } else {
      S.g[w] = s;
    }
  }
}

template <int BN>
__device__ void panel_reduce(const RqrArgs& a, int nbp, int ncx, RSmem<BN>& S);

// Panel block partials: P[k][c] = sum over my rows i >= j0 of conj(V(i,k)) X(i, c) with
// X = [V | M[:, c0:]] (the factorisation, with_gram) or X = M[:, c0:] (the Q formation).
template <int BN>
__device__ void panel_partials(const RqrArgs& a, const Rows& R, int j0, int nbp, int c0, int nct, bool with_gram,
                               RSmem<BN>& S) {
  const int G = gridDim.x, b = blockIdx.x;
  double* pp = a.scr + rq_off_pp(G) + (size_t)b * 2 * qpw<BN>();
  const int ng = with_gram ? nbp : 0;
  const int ncx = ng + nct;
  const long long lo = R.r0 > j0 ? R.r0 : j0;
  for (int e = threadIdx.x; e < nbp * ncx; e += QT) {
    const int k = e / ncx, c = e % ncx;
    double2 s0 = make_double2(0.0, 0.0), s1 = s0;
    long long i = lo;
    for (; i + 1 < R.r1; i += 2) {
      const double2 x0 = c < ng ? R.v(i, j0, c) : R.at(i, c0 + c - ng);
      const double2 x1 = c < ng ? R.v(i + 1, j0, c) : R.at(i + 1, c0 + c - ng);
      s0 = qfmac(s0, R.v(i, j0, k), x0);
      s1 = qfmac(s1, R.v(i + 1, j0, k), x1);
    }
    if (i < R.r1) s0 = qfmac(s0, R.v(i, j0, k), c < ng ? R.v(i, j0, c) : R.at(i, c0 + c - ng));
    const double2 s = qadd(s0, s1);
    if (G == 1) {
      S.P[k][c] = s;  // a single partial is the sum
    } else {
      pp[2 * e] = s.x;
      pp[2 * e + 1] = s.y;
    }
  }
}

// the panel block sums in S.P: one CTA has them already, several reduce their partials
template <int BN>
__device__ void panel_sums(const RqrArgs& a, int nbp, int ncx, RSmem<BN>& S) {
  if (gridDim.x == 1) {
    __syncthreads();
    return;
  }
  grid_barrier(a.bar, a.err);
  panel_reduce<BN>(a, nbp, ncx, S);
}

// every CTA sums a slice of the panel block entries over the G partials (one warp per
// entry), then, after a grid barrier, every CTA loads the whole block into S.P
template <int BN>
__device__ void panel_reduce(const RqrArgs& a, int nbp, int ncx, RSmem<BN>& S) {
  const int G = gridDim.x, b = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double* pp = a.scr + rq_off_pp(G);
  double* pr = a.scr + rq_off_pr<BN>(G);
  const int total = nbp * ncx;
  for (int e = b + G * warp; e < total; e += G * QW) {
    double sx = 0.0, sy = 0.0;
    for (int q = lane; q < G; q += 32) {
      sx += pp[(size_t)q * 2 * qpw<BN>() + 2 * e];
      sy += pp[(size_t)q * 2 * qpw<BN>() + 2 * e + 1];
    }
    const double2 t = warp_sum2(make_double2(sx, sy));
    sx = t.x;
    sy = t.y;
    if (lane == 0) {
      pr[2 * e] = sx;
      pr[2 * e + 1] = sy;
    }
  }
  grid_barrier(a.bar, a.err);
  for (int e = threadIdx.x; e < total; e += QT) S.P[e / ncx][e % ncx] = make_double2(pr[2 * e], pr[2 * e + 1]);
  __syncthreads();
}

// T of panel p from its Gram matrix S.P[:, 0:nbp] and the taus (zlarft forward,
// column-wise): T(i,i) = tau_i, T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i); one warp
template <int BN>
__device__ void form_t(int p, int j0, int nbp, RSmem<BN>& S) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    for (int i = 0; i < nbp; ++i) {
      const double2 ti = S.tau[j0 + i];
      double2 z = make_double2(0.0, 0.0);
      if (lane < i)
        z = make_double2(-(ti.x * S.P[lane][i].x - ti.y * S.P[lane][i].y),
                         -(ti.x * S.P[lane][i].y + ti.y * S.P[lane][i].x));
      __syncwarp();
      if (lane < QNB) S.W[0][lane] = z;  // scratch column
      __syncwarp();
      double2 t = make_double2(0.0, 0.0);
      if (lane < i)
        for (int k = lane; k < i; ++k) t = qadd(t, qmul(S.T[p][lane][k], S.W[0][k]));
      __syncwarp();
      if (lane < i) S.T[p][lane][i] = t;
      if (lane == i) S.T[p][i][i] = ti;
      if (lane > i && lane < QNB) S.T[p][lane][i] = make_double2(0.0, 0.0);
      __syncwarp();
    }
  }
  __syncthreads();
}

// bytes of RSmem<BN>, rounded up to 256: the rows start there
template <int BN> __host__ __device__ constexpr size_t rsmem_bytes() { return (sizeof(RSmem<BN>) + 255) / 256 * 256; }

template <int BN>
__global__ void __launch_bounds__(QT) k_qr_rows(RqrArgs a) {
  extern __shared__ __align__(256) unsigned char q_dyn[];
  RSmem<BN>& S = *reinterpret_cast<RSmem<BN>*>(q_dyn);
  double2* q_rows = reinterpret_cast<double2*>(q_dyn + rsmem_bytes<BN>());
  const int G = gridDim.x, b = blockIdx.x, n = a.n;
  const long long m = a.m;
  Rows R{q_rows, b * m / G, (b + 1) * m / G, n | 1};
  const int nr = (int)(R.r1 - R.r0);
  const double safmin = 2.2250738585072014e-308 / 1.1102230246251565e-16;
  const int npan = (n + QNB - 1) / QNB;
  QrClock pc{(a.phase && b == 0 && threadIdx.x == 0) ? a.phase : nullptr, 0ull};
  if (pc.acc) asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(pc.t));
  grid_barrier_begin(a.bar);
  for (int e = threadIdx.x; e < nr * n; e += QT) R.p[(e / n) * R.lds + e % n] = a.M[(R.r0 + e / n) * n + e % n];
  __syncthreads();
  col_partials<BN>(a, R, 0, n < QNB ? n : QNB, S);
  // ------------------------------------------------------------------ factorisation
  for (int p = 0; p < npan; ++p) {
    const int j0 = p * QNB, nbp = (n - j0) < QNB ? (n - j0) : QNB, jend = j0 + nbp;
    for (int j = j0; j < jend; ++j) {
      pc.mark(6);
      grid_barrier(a.bar, a.err);
      pc.mark(0);
      if (pc.acc) pc.acc[8] += 1;
      const int nc = jend - j - 1;
      col_reduce<BN>(a, j, jend, S);
      __syncthreads();
      pc.mark(1);
      if (threadIdx.x == 0) {
        const int E = S.E;
        double ar = S.rowj[0].x, ai = S.rowj[0].y;
        const double xn2 = S.nrm2, wa = fmax(fabs(ar), fabs(ai));
        int knt = 0;
        S.active = 0;
        if (E == 0 && xn2 > 1e-300 && xn2 < 1e300 && (wa == 0.0 || (wa > 1e-150 && wa < 1e150))) {
          // unscaled column of safe magnitude: beta from the squared norm by one square root,
          // tau and 1 / (alpha - beta) by one division each (independent of each other);
          // |beta| >= |x| > 1e-150, so no safe-minimum rescaling
          const double bb = -copysign(sqrt(fma(ar, ar, fma(ai, ai, xn2))), ar >= 0.0 ? 1.0 : -1.0);
          const double ib = 1.0 / bb;
          const double dr = ar - bb, di = ai;
          const double inv = 1.0 / fma(dr, dr, di * di);
          S.tau[j] = make_double2((bb - ar) * ib, -ai * ib);
          S.scal = make_double2(dr * inv, -di * inv);
          S.beta = make_double2(bb, 0.0);
          S.active = 1;
          S.kx = 0;
          S.kfac = 0;
          if (b == 0) a.tau_out[j] = S.tau[j];
        } else {
        double xnorm = sqrt(xn2);
        if (E) xnorm = qldexp(xnorm, E);
        if (xnorm == 0.0 && ai == 0.0) {
          S.tau[j] = make_double2(0.0, 0.0);
          S.beta = make_double2(ar, ai);
          S.scal = make_double2(0.0, 0.0);
        } else {
          // |(alpha, xnorm)| by one square root when no square can over- or underflow,
          // else by the scaled dlapy3 form
          const double w = fmax(fmax(fabs(ar), fabs(ai)), xnorm);
          const bool safe = w > 1e-150 && w < 1e150;
          double bb = -copysign(safe ? sqrt(fma(ar, ar, fma(ai, ai, xnorm * xnorm))) : qlapy3(ar, ai, xnorm),
                                ar >= 0.0 ? 1.0 : -1.0);
          if (fabs(bb) < safmin) {
            const double rs = 1.0 / safmin;
            do {
              ++knt;
              bb *= rs;
              ar *= rs;
              ai *= rs;
              xnorm *= rs;
            } while (fabs(bb) < safmin && knt < 20);
            bb = -copysign(qlapy3(ar, ai, xnorm), ar >= 0.0 ? 1.0 : -1.0);
          }
          S.tau[j] = make_double2((bb - ar) / bb, -ai / bb);
          // 1 / (alpha - beta): |alpha - beta| >= |beta|, so in the safe range the squared
          // magnitude is a normal number and one division suffices; else Smith's division
          const double dr = ar - bb, di = ai;
          if (fabs(bb) > 1e-150 && fabs(bb) < 1e150) {
            const double inv = 1.0 / fma(dr, dr, di * di);
            S.scal = make_double2(dr * inv, -di * inv);
          } else {
            S.scal = qdiv(make_double2(1.0, 0.0), make_double2(dr, di));
          }
          for (int q = 0; q < knt; ++q) bb *= safmin;
          S.beta = make_double2(bb, 0.0);
          S.active = 1;
        }
        // v_i = x_i 2^(969 knt) scal, so conj(v)^T x_c = conj(scal) 2^(969 knt + E) g_c
        S.kx = 969 * knt;
        S.kfac = 969 * knt + E;
        if (b == 0) a.tau_out[j] = S.tau[j];
        }
      }
      __syncthreads();
      pc.mark(2);
      if (threadIdx.x >= 1 && threadIdx.x <= nc) {
        // w_c = M[j][c] + conj(scal) 2^kfac g_c, times conj(tau)
        double2 t = qmulc(S.scal, S.g[threadIdx.x]);
        if (S.kfac) {
          t.x = qldexp(t.x, S.kfac);
          t.y = qldexp(t.y, S.kfac);
        }
        const double2 wc = qadd(S.rowj[threadIdx.x], t);
        S.w[threadIdx.x] = qmulc(S.tau[j], wc);
      }
      __syncthreads();
      pc.mark(3);
      // my rows: v below the diagonal, beta on it, the panel columns right of j updated
      if (S.active) {
        const double2 sc = S.scal;
        const int kx = S.kx;
        const long long lo = R.r0 > j + 1 ? R.r0 : j + 1;
        for (long long i = lo + threadIdx.x; i < R.r1; i += QT) {
          double2 x = R.at(i, j);
          if (kx) {
            x.x = qldexp(x.x, kx);
            x.y = qldexp(x.y, kx);
          }
          const double2 v = qmul(x, sc);
          R.at(i, j) = v;
          for (int c = 1; c <= nc; ++c) R.at(i, j + c) = qfms(R.at(i, j + c), v, S.w[c]);
        }
      }
      if (j >= R.r0 && j < R.r1 && threadIdx.x == 0) {
        R.at(j, j) = S.beta;
        if (S.active)
          for (int c = 1; c <= nc; ++c) R.at(j, j + c) = qfms(R.at(j, j + c), make_double2(1.0, 0.0), S.w[c]);
      }
      __syncthreads();
      pc.mark(4);
      if (j + 1 < jend) col_partials<BN>(a, R, j + 1, jend, S);
      pc.mark(5);
    }
    // ---- panel done: V top block for the Q formation, Gram and projections, T, update
    if (threadIdx.x < QNB * QNB) {
      const int aa = threadIdx.x / QNB, k = threadIdx.x % QNB;
      const long long i = j0 + aa;
      if (aa < nbp && k < nbp && i >= R.r0 && i < R.r1) {
        const double2 v = R.v(i, j0, k);
        double* vt = a.scr + rq_off_vt<BN>(G) + (size_t)p * 2 * QNB * QNB;
        vt[2 * (aa * QNB + k)] = v.x;
        vt[2 * (aa * QNB + k) + 1] = v.y;
      }
    }
    const int nct = n - jend;
    panel_partials<BN>(a, R, j0, nbp, jend, nct, true, S);
    panel_sums<BN>(a, nbp, nbp + nct, S);
    form_t<BN>(p, j0, nbp, S);
    if (nct > 0) {
      // W = T^H (V^H M_trailing)
      for (int e = threadIdx.x; e < nbp * nct; e += QT) {
        const int k = e / nct, c = e % nct;
        double2 s = make_double2(0.0, 0.0);
        for (int q = 0; q <= k; ++q) s = qfmac(s, S.T[p][q][k], S.P[q][nbp + c]);
        S.W[k][c] = s;
      }
      __syncthreads();
      const long long lo = R.r0 > j0 ? R.r0 : j0;
      for (long long e = threadIdx.x; e < (R.r1 - lo) * nct; e += QT) {
        const long long i = lo + e / nct;
        const int c = (int)(e % nct);
        double2 x = R.at(i, jend + c);
        for (int k = 0; k < nbp; ++k) x = qfms(x, R.v(i, j0, k), S.W[k][c]);
        R.at(i, jend + c) = x;
      }
      __syncthreads();
      col_partials<BN>(a, R, jend, jend + ((n - jend) < QNB ? (n - jend) : QNB), S);
    }
  }
  pc.mark(6);
  // ------------------------------------------------------------------ R
  for (int e = threadIdx.x; e < nr * n; e += QT) {
    const long long i = R.r0 + e / n;
    const int k = e % n;
    if (i >= n) continue;
    const double2 v = (k >= i) ? R.at(i, k) : make_double2(0.0, 0.0);
    if (a.Rt) a.R[(long long)k * n + i] = v;
    else a.R[i * n + k] = v;
  }
  grid_barrier(a.bar, a.err);  // the V top blocks of every panel are visible from here on
  // ------------------------------------------------------------------ Q, backwards
  for (int p = npan - 1; p >= 0; --p) {
    const int j0 = p * QNB, nbp = (n - j0) < QNB ? (n - j0) : QNB, jend = j0 + nbp;
    const int nct = n - jend;
    const long long lo = R.r0 > j0 ? R.r0 : j0;
    if (nct > 0) {
      panel_partials<BN>(a, R, j0, nbp, jend, nct, false, S);
      panel_sums<BN>(a, nbp, nct, S);
      // W = T (V^H Q_trailing); Q_trailing -= V W
      for (int e = threadIdx.x; e < nbp * nct; e += QT) {
        const int k = e / nct, c = e % nct;
        double2 s = make_double2(0.0, 0.0);
        for (int q = k; q < nbp; ++q) s = qadd(s, qmul(S.T[p][k][q], S.P[q][c]));
        S.W[k][c] = s;
      }
      __syncthreads();
      for (long long e = threadIdx.x; e < (R.r1 - lo) * nct; e += QT) {
        const long long i = lo + e / nct;
        const int c = (int)(e % nct);
        double2 x = R.at(i, jend + c);
        for (int k = 0; k < nbp; ++k) x = qfms(x, R.v(i, j0, k), S.W[k][c]);
        R.at(i, jend + c) = x;
      }
      __syncthreads();
    }
    // panel columns: Q[:, j0 + k] = e_{j0+k} - V W2, W2 = T V_top^H
    {
      const double* vt = a.scr + rq_off_vt<BN>(G) + (size_t)p * 2 * QNB * QNB;
      for (int e = threadIdx.x; e < nbp * nbp; e += QT) {
        const int aa = e / nbp, k = e % nbp;
        double2 s = make_double2(0.0, 0.0);
        for (int q = aa; q < nbp; ++q) {
          const double2 vkq = make_double2(vt[2 * (k * QNB + q)], vt[2 * (k * QNB + q) + 1]);  // V_top(k, q)
          s = qfmac(s, vkq, S.T[p][aa][q]);  // T(aa, q) conj(V_top(k, q))
        }
        S.W[aa][k] = s;
      }
      __syncthreads();
      for (long long i = R.r0 + threadIdx.x; i < R.r1; i += QT) {
        double2 v[QNB];
#pragma unroll
        for (int q = 0; q < QNB; ++q) v[q] = (q < nbp && i >= j0) ? R.v(i, j0, q) : make_double2(0.0, 0.0);
        for (int k = 0; k < nbp; ++k) {
          double2 x = make_double2(i == j0 + k ? 1.0 : 0.0, 0.0);
#pragma unroll
          for (int q = 0; q < QNB; ++q)
            if (q < nbp) x = qfms(x, v[q], S.W[q][k]);
          R.at(i, j0 + k) = x;
        }
      }
      __syncthreads();
    }
  }
  for (int e = threadIdx.x; e < nr * n; e += QT) a.M[(R.r0 + e / n) * n + e % n] = R.p[(e / n) * R.lds + e % n];
  __syncthreads();
  pc.mark(7);
  grid_barrier_end(a.bar);
}

template <int BN> size_t rows_smem(int rows, int n) { return rsmem_bytes<BN>() + (size_t)rows * (size_t)(n | 1) * sizeof(double2); }

// opt-in shared memory per block of the current device (the same for every GB300; looked
// up once)
int max_dyn_smem() {
  static int v = -1;
  if (v < 0) {
    int dev = 0, x = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&x, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    v = x;
  }
  return v;
}

// dynamic shared memory an instantiation may take: the opt-in limit less its static
// shared memory (the grid barrier's slot), which counts against the same limit
template <int BN> int dyn_limit() {
  static int v = -1;
  if (v < 0) {
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, k_qr_rows<BN>);
    v = max_dyn_smem() - (int)fa.sharedSizeBytes;
  }
  return v;
}

template <int BN> int rows_cap(int n) {
  const long long avail = (long long)dyn_limit<BN>() - (long long)rsmem_bytes<BN>();
  long long r = avail > 0 ? avail / ((long long)(n | 1) * (long long)sizeof(double2)) : 0;
  if (r > kQrRowsMax) r = kQrRowsMax;
  return (int)r;
}

template <int BN> int max_grid_bn() {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // every launch stays within the opt-in limit (rows_cap), whatever its width
  const int dyn = dyn_limit<BN>();
  cudaFuncSetAttribute(k_qr_rows<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_qr_rows<BN>, QT, dyn);
  return sms * (per < 1 ? 1 : per);
}

}  // namespace

size_t qr_rows_scratch_bytes(int max_grid) { return rq_doubles<kMaxBond>(max_grid) * sizeof(double); }

int qr_rows_max_rows(int n) { return n <= kQrMaxCols ? rows_cap<kQrMaxCols>(n) : rows_cap<kMaxBond>(n); }

int qr_rows_max_grid() {
  const int a = max_grid_bn<kQrMaxCols>(), b = max_grid_bn<kMaxBond>();
  return a < b ? a : b;
}

cudaError_t householder_qr_rows(double2* M, long long m, int n, double2* R, int Rt, double2* tau_ws, double* scratch,
                                GridBarrier* bar, int* err, int grid, cudaStream_t s, unsigned long long* phase) {
  if (n < 1 || n > kMaxBond || m < n || grid < 1 || grid > 32 * kQrPartsPerLane ||
      (m + grid - 1) / grid > qr_rows_max_rows(n))
    return cudaErrorInvalidValue;
  RqrArgs a{M, m, n, R, Rt, tau_ws, scratch, bar, err, phase};
  void* args[] = {&a};
  ++g_launches;
  const int rows = (int)((m + grid - 1) / grid);
  if (n <= kQrMaxCols)
    return cudaLaunchCooperativeKernel((const void*)k_qr_rows<kQrMaxCols>, dim3(grid), dim3(QT), args,
                                       rows_smem<kQrMaxCols>(rows, n), s);
  return cudaLaunchCooperativeKernel((const void*)k_qr_rows<kMaxBond>, dim3(grid), dim3(QT), args,
                                     rows_smem<kMaxBond>(rows, n), s);
}

}  // namespace ttn
