// Panel-blocked cooperative Householder QR of a tall complex matrix (m x n, n <= 64,
// row-major, in place): M <- Q (m x n), R (n x n) upper triangular, LAPACK zgeqrf /
// zungqr conventions (zlarfg reflectors: real beta, tau = (beta - alpha) / beta, v(1) = 1,
// scaled norms and the safe-minimum rescaling of tiny columns; H^H = I - conj(tau) v v^H
// applied from the left; Q = H_0 H_1 ... H_{n-1} [I; 0]).
//
// GB300 runs FP64 at 2 FMA/clk/SM with 64-cycle dependent latency, so the factorisation
// must use the whole device and the cost is the number of grid-wide synchronisations and
// the FP64 work around them.  The rows are split over the CTAs; per column j of a panel of
// NB columns there is ONE grid barrier: before it every CTA has published, for column j
// and its own rows, the scaled norm partial, the Gram products of column j with the later
// columns of the panel (scaled by a power of two so that nothing underflows) and, from the
// owner of row j, alpha and the rest of row j.  After it every CTA forms the reflector
// and the projections w_c = v^H M[:, c] for the panel columns from those sums alone,
// updates its rows and publishes the next column's partials.  The columns right of the
// panel are updated once per panel with the compact WY form H = I - V T V^H (zlarft,
// forward, column-wise; zlarfb), whose V^H [V | M] partials are reduced cooperatively
// (each CTA reduces a slice, then everyone reads the result).  Q is formed backwards panel
// by panel the same way (zungqr), the panel's own columns from H_p applied to identity
// columns without any reduction.
#include "ttn_coop.cuh"
#include "ttn_kernels.cuh"

#include <cstdint>

namespace ttn {
namespace {

constexpr int BT = 256;                 // threads per CTA
constexpr int NB = 8;                   // panel width
// BN: widest matrix of an instantiation (64, or kMaxBond); BN / NB panels at most;
// NB (NB + BN) complex entries in one panel block V^H [V | M_trailing]
template <int BN> __host__ __device__ constexpr int np_of() { return BN / NB; }
template <int BN> __host__ __device__ constexpr int pw_of() { return NB * (NB + BN); }

struct BqrArgs {
  double2* M;
  long long m;
  int n;
  double2* R;
  int Rt;
  double2* tau_out;
  double* scr;
  GridBarrier* bar;
  int* err;
};

// scratch layout (doubles), G = gridDim.x
__host__ __device__ constexpr size_t off_cp(int) { return 0; }                                   // [2][G][2]
__host__ __device__ constexpr size_t off_gp(int G) { return (size_t)4 * G; }                     // [2][G][2NB]
__host__ __device__ constexpr size_t off_cj(int G) { return off_gp(G) + (size_t)4 * NB * G; }    // [2][2+2NB]
__host__ __device__ constexpr size_t off_pp(int G) { return off_cj(G) + 2 * (2 + 2 * NB); }      // [G][2PW]
template <int BN> __host__ __device__ constexpr size_t off_pr(int G) { return off_pp(G) + (size_t)2 * pw_of<BN>() * G; }
template <int BN> __host__ __device__ constexpr size_t off_vt(int G) { return off_pr<BN>(G) + 2 * pw_of<BN>(); }
template <int BN> __host__ __device__ constexpr size_t scratch_doubles(int G) {
  return off_vt<BN>(G) + (size_t)np_of<BN>() * 2 * NB * NB;
}

__device__ __forceinline__ double2 cadd2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__device__ __forceinline__ double2 cmulc2(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 cfms(double2 c, double2 a, double2 b) {  // c - a * b
  c.x = fma(-a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(-a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ double2 cfmac(double2 c, double2 a, double2 b) {  // c + conj(a) * b
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}

// floor(log2(x)) for finite x > 0 (subnormals included), from the bits
__device__ __forceinline__ int ilog2_d(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e != 0) return e - 1023;
  const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  return -1074 + (63 - __clzll((long long)mant));
}
// x * 2^k, exact while the result is normal; |k| up to 2000 in two exact steps, scalings
// below 2^-2000 (contributions far below the rounding of the sums they enter) give 0
__device__ __forceinline__ double ldexp2(double x, int k) {
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
// max(|re|, |im|) through the bit patterns (non-negative doubles order like integers)
__device__ __forceinline__ unsigned long long absmax_bits(double2 v) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long b = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
  return a > b ? a : b;
}

__device__ double dlapy3_b(double x, double y, double z) {
  double w = fmax(fabs(x), fmax(fabs(y), fabs(z)));
  if (w == 0.0) return 0.0;
  double a = x / w, b = y / w, c = z / w;
  return w * sqrt(a * a + b * b + c * c);
}
__device__ double2 cdiv_b(double2 a, double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, den = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
  }
  double r = b.x / b.y, den = b.x * r + b.y;
  return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

template <int BN>
struct Smem {
  unsigned long long umax[BT / 32];
  double dsum[BT / 32];
  double2 csum[BT / 32][NB];
  double2 tau[BN];
  double2 T[BN / NB][NB][NB];  // compact WY factors of every panel
  double2 P[NB][NB + BN];    // reduced panel block (Gram | projections)
  double2 W[NB][NB + BN];    // T^H P (factorisation) or T P (Q formation)
  double2 w[NB];             // column projections within the panel (times conj(tau))
  double2 scal;              // 1 / (alpha - beta) in the rescaled units
  double2 beta;
  int kfac;                  // exponent of the factor between the Gram sums and w
  int active;
};

template <int BN>
__device__ __forceinline__ double block_sum_d(double v, Smem<BN>& S) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) S.dsum[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < BT / 32; ++k) s += S.dsum[k];
  __syncthreads();
  return s;
}
template <int BN>
__device__ __forceinline__ unsigned long long block_max_u(unsigned long long v, Smem<BN>& S) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t > v ? t : v;
  }
  if ((threadIdx.x & 31) == 0) S.umax[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long s = 0;
#pragma unroll
  for (int k = 0; k < BT / 32; ++k) s = S.umax[k] > s ? S.umax[k] : s;
  __syncthreads();
  return s;
}

// V(i, k) of panel [j0, j0 + nbp): 0 above the diagonal, 1 on it, M below
__device__ __forceinline__ double2 vpanel(const BqrArgs& a, long long i, int j0, int k) {
  const long long d = j0 + k;
  if (i < d) return make_double2(0.0, 0.0);
  if (i == d) return make_double2(1.0, 0.0);
  return a.M[i * a.n + d];
}

// Partials of column j for my rows (j < jend): scaled norm of rows > j, Gram of the
// subdiagonal part with the panel columns c in (j, jend), and from the owner of row j:
// alpha and M[j][c].
template <int BN>
__device__ void column_partials(const BqrArgs& a, int j, int jend, long long r0, long long r1, Smem<BN>& S) {
  const int G = gridDim.x, b = blockIdx.x, par = j & 1, n = a.n;
  double* cp = a.scr + off_cp(G) + (size_t)par * 2 * G;
  double* gp = a.scr + off_gp(G) + (size_t)par * 2 * NB * G;
  double* cj = a.scr + off_cj(G) + (size_t)par * (2 + 2 * NB);
  const long long lo = (r0 > j + 1) ? r0 : j + 1;
  unsigned long long um = 0;
  for (long long i = lo + threadIdx.x; i < r1; i += blockDim.x) {
    const unsigned long long t = absmax_bits(a.M[i * n + j]);
    um = t > um ? t : um;
  }
  um = block_max_u(um, S);
  const double lmax = __longlong_as_double((long long)um);
  const int eb = lmax > 0.0 ? ilog2_d(lmax) : 0;
  // scaled sum of squares and Gram products with x' = x 2^-eb; thread slots: c-index
  // (0..NB-1, 0 = the norm) x row subsets
  const int nc = jend - j - 1;
  const int slot = threadIdx.x % NB, sub = threadIdx.x / NB, nsub = BT / NB;
  double2 acc = make_double2(0.0, 0.0);
  if (lmax > 0.0) {
    for (long long i = lo + sub; i < r1; i += nsub) {
      double2 x = a.M[i * n + j];
      x.x = ldexp2(x.x, -eb);
      x.y = ldexp2(x.y, -eb);
      if (slot == 0) {
        acc.x = fma(x.x, x.x, acc.x);
        acc.x = fma(x.y, x.y, acc.x);
      } else if (slot <= nc) {
        acc = cfmac(acc, x, a.M[i * n + j + slot]);
      }
    }
  }
  // reduce over the row subsets: lanes with equal slot are 8 apart inside a warp
#pragma unroll
  for (int o = 16; o >= NB; o >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
  }
  if ((threadIdx.x & 31) < NB) S.csum[threadIdx.x >> 5][slot] = acc;
  __syncthreads();
  if (threadIdx.x < NB) {
    double2 s = make_double2(0.0, 0.0);
#pragma unroll
    for (int w = 0; w < BT / 32; ++w) s = cadd2(s, S.csum[w][threadIdx.x]);
    if (threadIdx.x == 0) {
      cp[2 * b] = lmax;
      cp[2 * b + 1] = s.x;
    } else if (threadIdx.x <= nc) {
      gp[(size_t)b * 2 * NB + 2 * threadIdx.x] = s.x;
      gp[(size_t)b * 2 * NB + 2 * threadIdx.x + 1] = s.y;
    }
  }
  if (j >= r0 && j < r1) {
    for (int c = threadIdx.x; c <= nc; c += blockDim.x) {
      const double2 v = a.M[(long long)j * n + j + c];
      cj[2 * c] = v.x;
      cj[2 * c + 1] = v.y;
    }
  }
  __syncthreads();
}

// Panel block partials: P[k][c] = sum over my rows i >= j0 of conj(V(i,k)) X(i, c) with
// X = [V | M[:, c0:]] (ncx = nbp + nct columns) for the factorisation, or X = M[:, c0:]
// (ncx = nct) for the Q formation.
template <int BN>
__device__ void panel_partials(const BqrArgs& a, int j0, int nbp, int c0, int nct, bool with_gram, long long r0,
                               long long r1) {
  const int G = gridDim.x, b = blockIdx.x, n = a.n;
  double* pp = a.scr + off_pp(G) + (size_t)b * 2 * pw_of<BN>();
  const int ncx = (with_gram ? nbp : 0) + nct;
  const long long lo = r0 > j0 ? r0 : j0;
  for (int e = threadIdx.x; e < nbp * ncx; e += blockDim.x) {
    const int k = e / ncx, c = e % ncx;
    double2 s0 = make_double2(0.0, 0.0), s1 = s0;
    long long i = lo;
    for (; i + 1 < r1; i += 2) {
      const double2 x0 = (with_gram && c < nbp) ? vpanel(a, i, j0, c) : a.M[i * n + c0 + c - (with_gram ? nbp : 0)];
      const double2 x1 =
          (with_gram && c < nbp) ? vpanel(a, i + 1, j0, c) : a.M[(i + 1) * n + c0 + c - (with_gram ? nbp : 0)];
      s0 = cfmac(s0, vpanel(a, i, j0, k), x0);
      s1 = cfmac(s1, vpanel(a, i + 1, j0, k), x1);
    }
    if (i < r1) {
      const double2 x0 = (with_gram && c < nbp) ? vpanel(a, i, j0, c) : a.M[i * n + c0 + c - (with_gram ? nbp : 0)];
      s0 = cfmac(s0, vpanel(a, i, j0, k), x0);
    }
    const double2 s = cadd2(s0, s1);
    pp[2 * e] = s.x;
    pp[2 * e + 1] = s.y;
  }
}

// every CTA reduces a slice of the panel block entries over the G partials (one warp
// per entry), then, after a barrier, every CTA loads the whole block into S.P
template <int BN>
__device__ void panel_reduce(const BqrArgs& a, int nbp, int ncx, Smem<BN>& S) {
  const int G = gridDim.x, b = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double* pp = a.scr + off_pp(G);
  double* pr = a.scr + off_pr<BN>(G);
  const int total = nbp * ncx;
  for (int e = b + G * warp; e < total; e += G * (BT / 32)) {
    double sx = 0.0, sy = 0.0;
    for (int q = lane; q < G; q += 32) {
      sx += pp[(size_t)q * 2 * pw_of<BN>() + 2 * e];
      sy += pp[(size_t)q * 2 * pw_of<BN>() + 2 * e + 1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if (lane == 0) {
      pr[2 * e] = sx;
      pr[2 * e + 1] = sy;
    }
  }
  grid_barrier(a.bar, a.err);
  for (int e = threadIdx.x; e < total; e += blockDim.x) S.P[e / ncx][e % ncx] = make_double2(pr[2 * e], pr[2 * e + 1]);
  __syncthreads();
}

// T of panel p from its Gram matrix S.P[:, 0:nbp] and the taus (zlarft forward,
// column-wise): T(i,i) = tau_i, T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i)
template <int BN>
__device__ void form_t(int p, int j0, int nbp, Smem<BN>& S) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    for (int i = 0; i < nbp; ++i) {
      const double2 ti = S.tau[j0 + i];
      double2 z = make_double2(0.0, 0.0);
      if (lane < i) z = make_double2(-(ti.x * S.P[lane][i].x - ti.y * S.P[lane][i].y),
                                     -(ti.x * S.P[lane][i].y + ti.y * S.P[lane][i].x));
      __syncwarp();
      if (lane < NB) S.W[0][lane] = z;  // scratch column
      __syncwarp();
      double2 t = make_double2(0.0, 0.0);
      if (lane < i)
        for (int k = lane; k < i; ++k) t = cadd2(t, cmul2(S.T[p][lane][k], S.W[0][k]));
      __syncwarp();
      if (lane < i) S.T[p][lane][i] = t;
      if (lane == i) S.T[p][i][i] = ti;
      if (lane > i && lane < NB) S.T[p][lane][i] = make_double2(0.0, 0.0);
      __syncwarp();
    }
  }
  __syncthreads();
}

template <int BN>
__global__ void __launch_bounds__(BT) k_qr_blocked(BqrArgs a) {
  extern __shared__ __align__(16) unsigned char b_dyn[];
  Smem<BN>& S = *reinterpret_cast<Smem<BN>*>(b_dyn);
  const int G = gridDim.x, b = blockIdx.x, n = a.n;
  const long long m = a.m;
  const long long r0 = b * m / G, r1 = (b + 1) * m / G;
  const double safmin = 2.2250738585072014e-308 / 1.1102230246251565e-16;
  const int npan = (n + NB - 1) / NB;
  grid_barrier_begin(a.bar);

  column_partials(a, 0, n < NB ? n : NB, r0, r1, S);
  // ------------------------------------------------------------------ factorisation
  for (int p = 0; p < npan; ++p) {
    const int j0 = p * NB, nbp = (n - j0) < NB ? (n - j0) : NB, jend = j0 + nbp;
    for (int j = j0; j < jend; ++j) {
      grid_barrier(a.bar, a.err);
      const int par = j & 1, nc = jend - j - 1;
      const double* cp = a.scr + off_cp(G) + (size_t)par * 2 * G;
      const double* gp = a.scr + off_gp(G) + (size_t)par * 2 * NB * G;
      const double* cj = a.scr + off_cj(G) + (size_t)par * (2 + 2 * NB);
      // global max of the column (scale 2^E) and sum of squares relative to it
      unsigned long long um = 0;
      for (int q = threadIdx.x; q < G; q += blockDim.x) {
        const unsigned long long t = (unsigned long long)__double_as_longlong(cp[2 * q]);
        um = t > um ? t : um;
      }
      um = block_max_u(um, S);
      const double amax = __longlong_as_double((long long)um);
      const int E = amax > 0.0 ? ilog2_d(amax) : 0;
      double ls = 0.0;
      for (int q = threadIdx.x; q < G; q += blockDim.x) {
        const double lm = cp[2 * q];
        if (lm > 0.0) ls += ldexp2(cp[2 * q + 1], 2 * (ilog2_d(lm) - E));
      }
      const double ssum = block_sum_d(ls, S);
      // Gram sums relative to 2^E: g_c = sum_b 2^(e_b - E) g'_b,c
      {
        const int slot = threadIdx.x % NB, sub = threadIdx.x / NB, nsub = BT / NB;
        double2 g = make_double2(0.0, 0.0);
        if (slot >= 1 && slot <= nc)
          for (int q = sub; q < G; q += nsub) {
            const double lm = cp[2 * q];
            if (lm > 0.0) {
              const int k = ilog2_d(lm) - E;
              g.x += ldexp2(gp[(size_t)q * 2 * NB + 2 * slot], k);
              g.y += ldexp2(gp[(size_t)q * 2 * NB + 2 * slot + 1], k);
            }
          }
#pragma unroll
        for (int o = 16; o >= NB; o >>= 1) {
          g.x += __shfl_xor_sync(0xffffffffu, g.x, o);
          g.y += __shfl_xor_sync(0xffffffffu, g.y, o);
        }
        if ((threadIdx.x & 31) < NB) S.csum[threadIdx.x >> 5][slot] = g;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double xnorm = ldexp2(sqrt(ssum), E);
        double ar = cj[0], ai = cj[1];
        int knt = 0;
        S.active = 0;
        if (xnorm == 0.0 && ai == 0.0) {
          S.tau[j] = make_double2(0.0, 0.0);
          S.beta = make_double2(ar, ai);
          S.scal = make_double2(0.0, 0.0);
        } else {
          // |(alpha, xnorm)| by one square root when no square can over- or underflow,
          // else by the scaled dlapy3 form
          const double w = fmax(fmax(fabs(ar), fabs(ai)), xnorm);
          const bool safe = w > 1e-150 && w < 1e150;
          double bb = -copysign(safe ? sqrt(fma(ar, ar, fma(ai, ai, xnorm * xnorm))) : dlapy3_b(ar, ai, xnorm),
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
            bb = -copysign(dlapy3_b(ar, ai, xnorm), ar >= 0.0 ? 1.0 : -1.0);
          }
          S.tau[j] = make_double2((bb - ar) / bb, -ai / bb);
          // 1 / (alpha - beta): |alpha - beta| >= |beta|, so in the safe range the squared
          // magnitude is a normal number and one division suffices; else Smith's division
          const double dr = ar - bb, di = ai;
          if (fabs(bb) > 1e-150 && fabs(bb) < 1e150) {
            const double inv = 1.0 / fma(dr, dr, di * di);
            S.scal = make_double2(dr * inv, -di * inv);
          } else {
            S.scal = cdiv_b(make_double2(1.0, 0.0), make_double2(dr, di));
          }
          for (int q = 0; q < knt; ++q) bb *= safmin;
          S.beta = make_double2(bb, 0.0);
          S.active = 1;
        }
        // v_i = x_i 2^(969 knt) scal, so conj(v)^T x_c = conj(scal) 2^(969 knt + E) g_c
        S.kfac = 969 * knt + E;
        if (b == 0) a.tau_out[j] = S.tau[j];
      }
      __syncthreads();
      const bool active = S.active != 0;
      const double2 tj = S.tau[j];
      const double2 sc = S.scal;
      const int kfac = S.kfac;
      const int kx = kfac - E;   // exponent of the rescaling of the column itself
      if (threadIdx.x >= 1 && threadIdx.x <= nc) {
        double2 g = make_double2(0.0, 0.0);
#pragma unroll
        for (int w = 0; w < BT / 32; ++w) g = cadd2(g, S.csum[w][threadIdx.x]);
        // w_c = M[j][c] + conj(scal) 2^kfac g_c, times conj(tau)
        double2 t = cmulc2(sc, g);
        t.x = ldexp2(t.x, kfac);
        t.y = ldexp2(t.y, kfac);
        const double2 wc = cadd2(make_double2(cj[2 * threadIdx.x], cj[2 * threadIdx.x + 1]), t);
        S.w[threadIdx.x] = cmulc2(tj, wc);
      }
      __syncthreads();
      // my rows: v below the diagonal, beta on it, panel columns right of j updated
      if (active) {
        const long long lo = r0 > j ? r0 : j;
        for (long long i = lo + threadIdx.x; i < r1; i += blockDim.x) {
          double2 v;
          if (i == j) {
            v = make_double2(1.0, 0.0);
          } else {
            double2 x = a.M[i * n + j];
            x.x = ldexp2(x.x, kx);
            x.y = ldexp2(x.y, kx);
            v = cmul2(x, sc);
            a.M[i * n + j] = v;
          }
          for (int c = 1; c <= nc; ++c) a.M[i * n + j + c] = cfms(a.M[i * n + j + c], v, S.w[c]);
        }
      }
      if (j >= r0 && j < r1 && threadIdx.x == 0) a.M[(long long)j * n + j] = S.beta;
      __syncthreads();
      if (j + 1 < jend) column_partials(a, j + 1, jend, r0, r1, S);
    }
    // ---- panel done: V top block for the Q formation, Gram and projections, T, update
    if (threadIdx.x < NB * NB) {
      const int aa = threadIdx.x / NB, k = threadIdx.x % NB;
      const long long i = j0 + aa;
      if (aa < nbp && k < nbp && i >= r0 && i < r1) {
        const double2 v = vpanel(a, i, j0, k);
        double* vt = a.scr + off_vt<BN>(G) + (size_t)p * 2 * NB * NB;
        vt[2 * (aa * NB + k)] = v.x;
        vt[2 * (aa * NB + k) + 1] = v.y;
      }
    }
    const int nct = n - jend;
    panel_partials<BN>(a, j0, nbp, jend, nct, true, r0, r1);
    grid_barrier(a.bar, a.err);
    panel_reduce(a, nbp, nbp + nct, S);
    form_t(p, j0, nbp, S);
    if (nct > 0) {
      // W = T^H (V^H M_trailing)
      for (int e = threadIdx.x; e < nbp * nct; e += blockDim.x) {
        const int k = e / nct, c = e % nct;
        double2 s = make_double2(0.0, 0.0);
        for (int q = 0; q <= k; ++q) s = cfmac(s, S.T[p][q][k], S.P[q][nbp + c]);
        S.W[k][c] = s;
      }
      __syncthreads();
      const long long lo = r0 > j0 ? r0 : j0;
      for (long long e = threadIdx.x; e < (r1 - lo) * nct; e += blockDim.x) {
        const long long i = lo + e / nct;
        const int c = (int)(e % nct);
        double2 x = a.M[i * n + jend + c];
        for (int k = 0; k < nbp; ++k) x = cfms(x, vpanel(a, i, j0, k), S.W[k][c]);
        a.M[i * n + jend + c] = x;
      }
      __syncthreads();
      column_partials(a, jend, jend + ((n - jend) < NB ? (n - jend) : NB), r0, r1, S);
    }
  }
  // ------------------------------------------------------------------ R
  for (long long e = threadIdx.x; e < (r1 - r0) * n; e += blockDim.x) {
    const long long i = r0 + e / n;
    const int k = (int)(e % n);
    if (i >= n) continue;
    const double2 v = (k >= i) ? a.M[i * n + k] : make_double2(0.0, 0.0);
    if (a.Rt) a.R[(long long)k * n + i] = v;
    else a.R[i * n + k] = v;
  }
  grid_barrier(a.bar, a.err);  // the V top blocks of every panel are visible from here on
  // ------------------------------------------------------------------ Q, backwards
  for (int p = npan - 1; p >= 0; --p) {
    const int j0 = p * NB, nbp = (n - j0) < NB ? (n - j0) : NB, jend = j0 + nbp;
    const int nct = n - jend;
    const long long lo = r0 > j0 ? r0 : j0;
    if (nct > 0) {
      panel_partials<BN>(a, j0, nbp, jend, nct, false, r0, r1);
      grid_barrier(a.bar, a.err);
      panel_reduce(a, nbp, nct, S);
      // W = T (V^H Q_trailing); Q_trailing -= V W
      for (int e = threadIdx.x; e < nbp * nct; e += blockDim.x) {
        const int k = e / nct, c = e % nct;
        double2 s = make_double2(0.0, 0.0);
        for (int q = k; q < nbp; ++q) s = cadd2(s, cmul2(S.T[p][k][q], S.P[q][c]));
        S.W[k][c] = s;
      }
      __syncthreads();
      for (long long e = threadIdx.x; e < (r1 - lo) * nct; e += blockDim.x) {
        const long long i = lo + e / nct;
        const int c = (int)(e % nct);
        double2 x = a.M[i * n + jend + c];
        for (int k = 0; k < nbp; ++k) x = cfms(x, vpanel(a, i, j0, k), S.W[k][c]);
        a.M[i * n + jend + c] = x;
      }
      __syncthreads();
    }
    // panel columns: Q[:, j0 + k] = e_{j0+k} - V W2, W2 = T V_top^H
    {
      const double* vt = a.scr + off_vt<BN>(G) + (size_t)p * 2 * NB * NB;
      for (int e = threadIdx.x; e < nbp * nbp; e += blockDim.x) {
        const int aa = e / nbp, k = e % nbp;
        double2 s = make_double2(0.0, 0.0);
        for (int q = aa; q < nbp; ++q) {
          const double2 vkq = make_double2(vt[2 * (k * NB + q)], vt[2 * (k * NB + q) + 1]);  // V_top(k, q)
          s = cfmac(s, vkq, S.T[p][aa][q]);  // T(aa, q) conj(V_top(k, q))
        }
        S.W[aa][k] = s;
      }
      __syncthreads();
      for (long long i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
        double2 v[NB];
#pragma unroll
        for (int q = 0; q < NB; ++q) v[q] = (q < nbp && i >= j0) ? vpanel(a, i, j0, q) : make_double2(0.0, 0.0);
        for (int k = 0; k < nbp; ++k) {
          double2 x = make_double2(i == j0 + k ? 1.0 : 0.0, 0.0);
#pragma unroll
          for (int q = 0; q < NB; ++q)
            if (q < nbp) x = cfms(x, v[q], S.W[q][k]);
          a.M[i * n + j0 + k] = x;
        }
      }
      __syncthreads();
    }
  }
  grid_barrier_end(a.bar);
}

}  // namespace

size_t qr_blocked_scratch_bytes(int max_grid) { return scratch_doubles<kMaxBond>(max_grid) * sizeof(double); }

namespace {
template <int BN> int blocked_max_grid_bn() {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(k_qr_blocked<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem<BN>));
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_qr_blocked<BN>, BT, sizeof(Smem<BN>));
  return sms * (per < 1 ? 1 : per);
}
}  // namespace

int qr_blocked_max_grid() {
  const int a = blocked_max_grid_bn<kQrMaxCols>(), b = blocked_max_grid_bn<kMaxBond>();
  return a < b ? a : b;
}

cudaError_t householder_qr_blocked(double2* M, long long m, int n, double2* R, int Rt, double2* tau_ws,
                                   double* scratch, GridBarrier* bar, int* err, int grid, cudaStream_t s) {
  if (n < 1 || n > kMaxBond || m < n || grid < 1) return cudaErrorInvalidValue;
  BqrArgs a{M, m, n, R, Rt, tau_ws, scratch, bar, err};
  void* args[] = {&a};
  ++g_launches;
  if (n <= kQrMaxCols)
    return cudaLaunchCooperativeKernel((const void*)k_qr_blocked<kQrMaxCols>, dim3(grid), dim3(BT), args,
                                       sizeof(Smem<kQrMaxCols>), s);
  return cudaLaunchCooperativeKernel((const void*)k_qr_blocked<kMaxBond>, dim3(grid), dim3(BT), args,
                                     sizeof(Smem<kMaxBond>), s);
}

}  // namespace ttn
