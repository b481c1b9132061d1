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
constexpr int kSliceReduceGrid = 64;  // from this many CTAs on, coefficient sums are split over CTAs

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

// one contraction of the matvec program over all output elements (grid-stride), one
// thread per output element (the element-wise form; a.tpo == 1)
__device__ void run_op_1(const ExpmArgs& a, const MvOp& op, const double2* x) {
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
      // four independent chains: FP64 latency, not throughput, bounds small contractions;
      // the operands of eight steps are loaded before they are used
      double2 s0 = make_double2(0.0, 0.0), s1 = s0, s2 = s0, s3 = s0;
      int j = 0;
      for (; j + 8 <= d; j += 8) {
        double2 sa[8], va[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          sa[u] = S[j + u];
          va[u] = v[(long long)(j + u) * nb];
        }
        s0 = cfma(sa[0], va[0], s0);
        s1 = cfma(sa[1], va[1], s1);
        s2 = cfma(sa[2], va[2], s2);
        s3 = cfma(sa[3], va[3], s3);
        s0 = cfma(sa[4], va[4], s0);
        s1 = cfma(sa[5], va[5], s1);
        s2 = cfma(sa[6], va[6], s2);
        s3 = cfma(sa[7], va[7], s3);
      }
      for (; j < d; ++j) s0 = cfma(S[j], v[(long long)j * nb], s0);
      const double2 s = cadd(cadd(s0, s1), cadd(s2, s3));
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
      double2 s0 = make_double2(0.0, 0.0), s1 = s0, s2 = s0, s3 = s0;
      int l = 0;
      for (; l + 8 <= r; l += 8) {
        double2 va[8], ma[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          va[u] = v[l + u];
          ma[u] = M[l + u];
        }
        s0 = cfma(va[0], ma[0], s0);
        s1 = cfma(va[1], ma[1], s1);
        s2 = cfma(va[2], ma[2], s2);
        s3 = cfma(va[3], ma[3], s3);
        s0 = cfma(va[4], ma[4], s0);
        s1 = cfma(va[5], ma[5], s1);
        s2 = cfma(va[6], ma[6], s2);
        s3 = cfma(va[7], ma[7], s3);
      }
      for (; l < r; ++l) s0 = cfma(v[l], M[l], s0);
      const double2 s = cadd(cadd(s0, s1), cadd(s2, s3));
      double2 o = cmul(op.alpha, s);
      if (acc) o = cadd(o, out[e]);
      out[e] = o;
    }
  } else if (op.kind == MV_CSR) {
    const int d = op.d;
    const long long nb = op.nb, total = op.na * d * nb;
    for (long long e = tid; e < total; e += nthreads) {
      const long long aa = e / (d * nb), rem = e % (d * nb);
      const int i = (int)(rem / nb);
      const long long b = rem % nb;
      const double2* v = in + aa * d * nb + b;
      double2 s0 = make_double2(0.0, 0.0), s1 = s0;
      int q = op.rowptr[i];
      const int q1 = op.rowptr[i + 1];
      for (; q + 2 <= q1; q += 2) {
        s0 = cfma(op.mat[q], v[(long long)op.colind[q] * nb], s0);
        s1 = cfma(op.mat[q + 1], v[(long long)op.colind[q + 1] * nb], s1);
      }
      if (q < q1) s0 = cfma(op.mat[q], v[(long long)op.colind[q] * nb], s0);
      double2 r = cmul(op.alpha, cadd(s0, s1));
      if (acc) r = cadd(r, out[e]);
      out[e] = r;
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

// The same contraction with a.tpo (2, 4 or 8) consecutive lanes per output element: the
// lanes of a group take every tpo-th term of the sum and combine their partial sums by
// shuffles, and the group's first lane writes the element.  Small programs (leaves, bond
// matrices, medium nodes) have far fewer output elements than the launch has threads and
// are bound by the latency of one thread's chain of loads and FMAs, which this divides by
// tpo.  Every op of a program uses the same groups, so the thread that writes element e
// is the same in every op (accumulations into one buffer need no barrier between them);
// the Lanczos passes own elements by thread, so such a program ends with a grid barrier.
__device__ void run_op_g(const ExpmArgs& a, const MvOp& op, const double2* x) {
  const double2* in = buf_of(a, op.in, x);
  double2* out = buf_of(a, op.out, x);
  const int tpo = a.tpo;
  const long long nthreads = (long long)gridDim.x * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ngroups = nthreads / tpo, group = tid / tpo;
  const int part = (int)(tid % tpo);
  const bool acc = (op.beta != 0);
  long long total;
  if (op.kind == MV_MODE || op.kind == MV_CSR) total = op.na * op.d * op.nb;
  else if (op.kind == MV_MF) total = op.na * op.d;
  else total = op.na;
  // uniform trip count across the warp: every lane joins the shuffles
  for (long long e0 = 0; e0 < total; e0 += ngroups) {
    const long long e = e0 + group;
    const bool live = e < total;
    double2 s = make_double2(0.0, 0.0);
    if (op.kind == MV_MODE) {
      if (live) {
        const int d = op.d;
        const long long nb = op.nb;
        const long long aa = e / (d * nb), rem = e % (d * nb);
        const int i = (int)(rem / nb);
        const long long b = rem % nb;
        const double2* S = op.mat + (long long)i * d;
        const double2* v = in + aa * d * nb + b;
        double2 s1 = s;
        int j = part;
        for (; j + tpo < d; j += 2 * tpo) {
          const double2 p0 = S[j], q0 = v[(long long)j * nb], p1 = S[j + tpo], q1 = v[(long long)(j + tpo) * nb];
          s = cfma(p0, q0, s);
          s1 = cfma(p1, q1, s1);
        }
        if (j < d) s = cfma(S[j], v[(long long)j * nb], s);
        s = cadd(s, s1);
      }
    } else if (op.kind == MV_MF) {
      if (live) {
        const int r = op.d;
        const long long xx = e / r;
        const int k = (int)(e % r);
        const double2* v = in + xx * r;
        const double2* M = op.mat + (long long)k * r;
        double2 s1 = s;
        int l = part;
        for (; l + tpo < r; l += 2 * tpo) {
          s = cfma(v[l], M[l], s);
          s1 = cfma(v[l + tpo], M[l + tpo], s1);
        }
        if (l < r) s = cfma(v[l], M[l], s);
        s = cadd(s, s1);
      }
    } else if (op.kind == MV_CSR) {
      if (live && part == 0) {
        const int d = op.d;
        const long long nb = op.nb;
        const long long aa = e / (d * nb), rem = e % (d * nb);
        const int i = (int)(rem / nb);
        const long long b = rem % nb;
        const double2* v = in + aa * d * nb + b;
        for (int q = op.rowptr[i]; q < op.rowptr[i + 1]; ++q) s = cfma(op.mat[q], v[(long long)op.colind[q] * nb], s);
      }
    }
    if (op.kind == MV_MODE || op.kind == MV_MF) {
      for (int o = tpo >> 1; o > 0; o >>= 1) {
        s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
        s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
      }
    }
    if (live && part == 0) {
      double2 r;
      if (op.kind == MV_AXPY) r = cmul(op.alpha, in[e]);
      else if (op.kind == MV_ZERO) r = make_double2(0.0, 0.0);
      else r = cmul(op.alpha, s);
      if (acc && op.kind != MV_ZERO) r = cadd(r, out[e]);
      out[e] = r;
    }
  }
}

__device__ __forceinline__ void run_op(const ExpmArgs& a, const MvOp& op, const double2* x) {
  if (a.tpo > 1) run_op_g(a, op, x);
  else run_op_1(a, op, x);
}

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// wall time per phase as seen by one thread of CTA 0 (barrier waits included)
struct PhaseClock {
  unsigned long long* acc;
  unsigned long long t;
  __device__ void mark(int k) {
    if (acc) {
      const unsigned long long now = gtimer();
      acc[k] += now - t;
      t = now;
    }
  }
};

// ---- tensor-core contractions (mixed precision) at FP64 accuracy
//
// Both kinds are D(128 x N) = A B^T per tile (N = kTcTileN = 32), A the real block form
// of alpha * mat (64 x 64, row = output index, column = input index) and B N input
// columns n:
//   MODE tile (aa, b0): in(aa, j, b0 + n);   MF tile x0: in(x0 + n, j)   (j < 64)
// (32 columns per tile, not 64: a 4096 x 64 node's contractions then have 128 tiles for the
// 152 SMs instead of 64, and the per-tile B slicing, TMEM drain and output halve)
// with K = 128 ordered k = 2 j + c (c = 0 real, 1 imaginary part of input j):
//   A[(0,i)][(j,0)] = Re S, A[(0,i)][(j,1)] = -Im S, A[(1,i)][(j,0)] = Im S, A[(1,i)][(j,1)] = Re S.
// Exact integer slices (the Ozaki splitting): every row of A and of B is scaled by a power
// of two 2^E (E the smallest with all |x| < 2^E) and cut into six 7-bit integer slices,
// x = 2^E sum_t s_t 2^(-7t) + O(2^(E-42)), each slice exact in TF32.  The products s_t s_u
// (< 2^14) summed over K = 128 and over the at most 7 pairs of one level L = t + u stay
// below 2^24, so each level is accumulated EXACTLY in FP32 TMEM (levels 2..8, 7 x N
// columns); the epilogue combines the levels in integers and scales by 2^(E_i + E_n - 56).
// Error: the 42-bit truncation of the operands and the dropped levels >= 9, about 1e-13
// relative to sum_k |A||B| (FP64 contractions: about 1e-16).  Operands arrive in 4 chunks
// of 32 k (A: 6 slices x 16 KB by one bulk copy from the per-launch operator image; B:
// sliced from the FP64 vector on the integer pipe), 104 MMAs per chunk.
struct TcState {
  uint32_t tmem;          // TMEM base (512 columns)
  uint32_t mph[2];        // MMA mbarrier parities
  uint32_t lph[2];        // bulk-load mbarrier parities
  uint64_t* mbar;         // [2] MMA completion, one per operand buffer
  uint64_t* lbar;         // [2] bulk-load completion
  unsigned char* a[2];    // A chunk buffers: 6 slices x 128 x 32 bf16; both together the epilogue stage
  unsigned char* b[2];    // B chunk buffers: 6 slices x N x 32 bf16
  int* e_n;               // row exponents of the B tile
};
constexpr int TC_SLICES = 6;
constexpr int TC_LEVELS = 7;                              // t + u = 2 .. 8
constexpr int TC_CHUNK_K = 32;
constexpr int TC_CHUNKS = 4;
constexpr int TC_A_SLICE_BYTES = 128 * TC_CHUNK_K * 2;    // 8 KB
constexpr int TC_N = kTcTileN;                            // columns per tile
constexpr int TC_B_SLICE_BYTES = TC_N * TC_CHUNK_K * 2;   // 2 KB
constexpr int TC_A_CHUNK_BYTES = TC_SLICES * TC_A_SLICE_BYTES;
constexpr int TC_B_CHUNK_BYTES = TC_SLICES * TC_B_SLICE_BYTES;
constexpr int TC_IMG_HDR = 1024;                          // int E_i[64], padded
constexpr int TC_STAGE_LD = 65;                           // doubles per staged row
constexpr size_t TC_SMEM = (size_t)2 * (TC_A_CHUNK_BYTES + TC_B_CHUNK_BYTES) + 256;
constexpr uint32_t TC_TMEM_COLS = 256;
static_assert(kTcImageBytes == (size_t)TC_IMG_HDR + (size_t)TC_CHUNKS * TC_A_CHUNK_BYTES, "image size");
static_assert(128 * TC_STAGE_LD * 8 <= 2 * TC_A_CHUNK_BYTES, "epilogue stage must fit in the A buffers");
static_assert(TC_LEVELS * TC_N <= (int)TC_TMEM_COLS, "TMEM columns");
static_assert(TC_N % 16 == 0 && TC_N >= 16 && TC_N <= 64, "MMA N for M = 128");

// smallest E with |x| < 2^E from the bits of |x| (x != 0)
__device__ __forceinline__ int exp_bound_bits(unsigned long long absbits) {
  const int e = (int)(absbits >> 52);
  if (e != 0) return e - 1022;
  return -1074 + (64 - __clzll((long long)absbits));
}
// the six 7-bit slices of x relative to 2^Er (|x| < 2^Er), with the sign of x, as bf16
// (integers of at most 7 bits are exact in bf16)
__device__ __forceinline__ void slice6(double x, int Er, uint32_t* w) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long frac = b & 0xFFFFFFFFFFFFFull;
  unsigned long long q = 0;
  if (e != 0 || frac != 0) {
    const unsigned long long m = e ? (frac | (1ull << 52)) : frac;
    const int p = e ? e - 1075 : -1074;          // |x| = m 2^p
    const int sh = Er - 42 - p;                  // q = floor(|x| 2^(42 - Er)) < 2^42
    q = sh >= 64 ? 0ull : (sh >= 0 ? (m >> sh) : (m << (-sh)));
  }
  const uint32_t sgn = (uint32_t)(b >> 63) << 15;
#pragma unroll
  for (int t = 0; t < TC_SLICES; ++t) {
    const uint32_t v = (uint32_t)((q >> (35 - 7 * t)) & 127ull);
    // (float)v exactly: 2^23 + v has v in its low mantissa bits; subtracting 2^23 is exact
    const float f = __uint_as_float(0x4B000000u | v) - 8388608.0f;
    w[t] = (__float_as_uint(f) >> 16) | (v ? sgn : 0u);
  }
}
// the integer held exactly by an FP32 accumulator (|x| < 2^24), from its bits
__device__ __forceinline__ long long f32_exact_int(float x) {
  const uint32_t b = __float_as_uint(x);
  const int e = (int)((b >> 23) & 0xFF);
  if (e < 127) return 0;  // |x| < 1 is 0 for an integer
  const uint32_t m = (b & 0x7FFFFFu) | 0x800000u;
  const long long v = (long long)(m >> (150 - e));  // e <= 150 since |x| < 2^24
  return (b >> 31) ? -v : v;
}
// v * 2^e2 as a double from integer operations (truncating below 53 bits; 0 below the
// normal range)
__device__ __forceinline__ double i64_to_scaled_double(long long v, int e2) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
  const unsigned long long a = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
  const int msb = 63 - __clzll((long long)a);
  const unsigned long long mant = msb > 52 ? (a >> (msb - 52)) : (a << (52 - msb));
  const int ex = msb + e2 + 1023;
  if (ex <= 0) return 0.0;
  if (ex >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)ex << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// operator images of every tensor-core op of the program (all CTAs, one warp per row i):
// [int E_i[64]] then 4 chunks x 6 slices of the 128 x 32 bf16 operand, k = 2 j + c packed
// in pairs (real, imaginary input part) per 32-bit word
__device__ void build_tc_images(const ExpmArgs& a) {
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
  const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  int ntc = 0;
  for (int k = 0; k < a.nops; ++k) ntc += a.prog[k].tc ? 1 : 0;
  for (long long task = gw; task < (long long)ntc * 64; task += nwarps) {
    int which = (int)(task / 64);
    const int i = (int)(task % 64);
    const MvOp* opp = nullptr;
    for (int k = 0; k < a.nops; ++k)
      if (a.prog[k].tc && which-- == 0) {
        opp = &a.prog[k];
        break;
      }
    const MvOp& op = *opp;
    unsigned char* img = reinterpret_cast<unsigned char*>(a.tc_img) + (size_t)op.img * kTcImageBytes;
    double2 sv[2];
    unsigned long long mx = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      sv[h] = cmul(op.alpha, op.mat[i * 64 + lane + 32 * h]);
      const unsigned long long ar = (unsigned long long)__double_as_longlong(sv[h].x) & 0x7FFFFFFFFFFFFFFFull;
      const unsigned long long ai = (unsigned long long)__double_as_longlong(sv[h].y) & 0x7FFFFFFFFFFFFFFFull;
      mx = ar > mx ? ar : mx;
      mx = ai > mx ? ai : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = t > mx ? t : mx;
    }
    const int Er = mx ? exp_bound_bits(mx) : 0;
    if (lane == 0) reinterpret_cast<int*>(img)[i] = Er;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j = lane + 32 * h;
      const int q = j / 16, kc = 2 * (j % 16);
      unsigned char* chunk = img + TC_IMG_HDR + (size_t)q * TC_A_CHUNK_BYTES;
      uint32_t wr[TC_SLICES], wi[TC_SLICES], wn[TC_SLICES];
      slice6(sv[h].x, Er, wr);
      slice6(sv[h].y, Er, wi);
      slice6(-sv[h].y, Er, wn);
#pragma unroll
      for (int t = 0; t < TC_SLICES; ++t) {
        unsigned char* sl = chunk + t * TC_A_SLICE_BYTES;
        *reinterpret_cast<uint32_t*>(sl + tc::b16_offset(i, kc, 128)) = wr[t] | (wn[t] << 16);       // re out
        *reinterpret_cast<uint32_t*>(sl + tc::b16_offset(64 + i, kc, 128)) = wi[t] | (wr[t] << 16);  // im out
      }
    }
  }
  // the images are read by bulk copies (async proxy) after the next grid barrier
  tc::fence_proxy_async_all();
}

// row exponents of the B tile: 256 / N threads per row n, 64 N / 256 inputs each
__device__ __forceinline__ void tc_b_exponents(const TcState& t, const double2* base, long long sn, long long sj) {
  constexpr int TPR = 256 / TC_N, JPT = 64 / TPR;
  const int n = threadIdx.x / TPR, part = threadIdx.x % TPR;
  unsigned long long mx = 0;
  if (n < TC_N) {
#pragma unroll
    for (int j = JPT * part; j < JPT * part + JPT; ++j) {
      const double2 v = base[(long long)n * sn + (long long)j * sj];
      const unsigned long long ar = (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
      const unsigned long long ai = (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
      mx = ar > mx ? ar : mx;
      mx = ai > mx ? ai : mx;
    }
  }
#pragma unroll
  for (int o = 1; o < TPR; o <<= 1) {
    const unsigned long long u = __shfl_xor_sync(0xffffffffu, mx, o);
    mx = u > mx ? u : mx;
  }
  if (n < TC_N && part == 0) t.e_n[n] = mx ? exp_bound_bits(mx) : 0;
  __syncthreads();
}

// slices of chunk q of the B tile (inputs j = 16 q .. 16 q + 15) into buffer bi
// (tensor-core programs run with 256 threads: N / 16 rounds of 256 (n, jj) tasks; the
// lanes of a warp cover one 8-row x 4-word block of core matrices, 128 contiguous bytes per
// slice store, so the stores are free of bank conflicts)
__device__ __forceinline__ void tc_stage_b(const TcState& t, int bi, const double2* base, long long sn, long long sj,
                                           int q) {
  constexpr int NBLK = TC_N / 8;  // 8-row blocks of the tile
#pragma unroll
  for (int r = 0; r < TC_N / 16; ++r) {
    const int task = threadIdx.x + 256 * r;
    const int blk = task >> 5, ln = task & 31;
    const int n = (blk % NBLK) * 8 + (ln >> 2), jj = (blk / NBLK) * 4 + (ln & 3);
    const double2 v = base[(long long)n * sn + (long long)(16 * q + jj) * sj];
    const int Er = t.e_n[n];
    uint32_t wr[TC_SLICES], wi[TC_SLICES];
    slice6(v.x, Er, wr);
    slice6(v.y, Er, wi);
    const uint32_t o = tc::b16_offset(n, 2 * jj, TC_N);
#pragma unroll
    for (int s = 0; s < TC_SLICES; ++s)
      *reinterpret_cast<uint32_t*>(t.b[bi] + s * TC_B_SLICE_BYTES + o) = wr[s] | (wi[s] << 16);
  }
}

// issue the MMAs of chunk q from buffer bi (26 slice pairs x 2 k-steps) and commit them
// to mbar[bi]; one thread.  A descriptor's start address is its low 14 bits in 16-byte
// units, so every operand slice's descriptor is the buffer's plus a constant.
__device__ __forceinline__ void tc_issue_chunk(const TcState& t, int q, int bi) {
  const uint32_t idesc = tc::idesc_bf16(128, TC_N);
  const uint64_t ad0 = tc::smem_desc(tc::smem_u32(t.a[bi]), 16 * 128, 128);
  const uint64_t bd0 = tc::smem_desc(tc::smem_u32(t.b[bi]), (TC_N / 8) * 128, 128);
#pragma unroll
  for (int kk = 0; kk < TC_CHUNK_K / 16; ++kk) {
#pragma unroll
    for (int s = 0; s < TC_SLICES; ++s)
#pragma unroll
      for (int u = 0; u < TC_SLICES; ++u) {
        const int L = s + u;  // level - 2
        if (L >= TC_LEVELS) continue;
        const uint64_t ad = ad0 + (uint64_t)((s * TC_A_SLICE_BYTES + kk * 2 * 16 * 128) >> 4);
        const uint64_t bd = bd0 + (uint64_t)((u * TC_B_SLICE_BYTES + kk * 2 * (TC_N / 8) * 128) >> 4);
        // the first product into a level starts it: chunk 0, k-step 0, smallest s of the level
        const bool first = (q == 0 && kk == 0 && (s == (L < TC_SLICES ? 0 : L - TC_SLICES + 1)));
        tc::mma_bf16(t.tmem + (uint32_t)TC_N * (uint32_t)L, ad, bd, idesc, first ? 0u : 1u);
      }
  }
  tc::mma_commit(&t.mbar[bi]);
}

__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t& ph) {
  const bool ok = tc::mbar_wait(bar, ph);
  ph ^= 1u;
  return ok;
}

// TMEM -> stage (double [128][TC_STAGE_LD] over the A buffers): warp w drains TMEM lanes
// 32 (w % 4) .. + 31 (one row each), columns (N / 2) (w / 4) .. + N / 2 - 1; exact integer
// combination of the 7 levels, scaled by 2^(E_i + E_n - 56)
__device__ __forceinline__ void tc_drain_to_stage(const TcState& t, int Ei, PhaseClock& pc) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row_i = 32 * (warp & 3) + lane;
  double* row = reinterpret_cast<double*>(t.a[0]) + row_i * TC_STAGE_LD;
  const uint32_t lane_base = t.tmem + ((uint32_t)(32 * (warp & 3)) << 16);
  for (int c0 = (TC_N / 2) * (warp >> 2); c0 < (TC_N / 2) * (warp >> 2) + TC_N / 2; c0 += 8) {
    float f[TC_LEVELS][8];
#pragma unroll
    for (int L = 0; L < TC_LEVELS; ++L) tc::tmem_ld8_nowait(lane_base + (uint32_t)TC_N * L + (uint32_t)c0, f[L]);
    tc::tmem_wait_ld();
    pc.mark(15);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      // sum_L acc_L 2^(7 (6 - L)) / 2: levels 2,3 shifted by 34, the rest below; the bit
      // dropped is 2^-57 of the scale
      const long long hi = f32_exact_int(f[0][c]) * 128 + f32_exact_int(f[1][c]);
      long long lo = 0;
#pragma unroll
      for (int L = 2; L < TC_LEVELS; ++L) lo += f32_exact_int(f[L][c]) << (7 * (TC_LEVELS - 1 - L));
      const int e2 = Ei + t.e_n[c0 + c] - 56;
      row[c0 + c] = i64_to_scaled_double((hi << 34) + (lo >> 1), e2 + 1);
    }
  }
  tc::fence_before();
  __syncthreads();
}

__device__ void run_op_tc(const ExpmArgs& a, const MvOp& op, const double2* x, TcState& t) {
  const double2* in = buf_of(a, op.in, x);
  double2* out = buf_of(a, op.out, x);
  const bool acc = (op.beta != 0);
  const bool mode = (op.kind == MV_MODE);
  const long long nb = op.nb;
  const long long tiles = mode ? op.na * (nb / TC_N) : op.na / TC_N;
  if ((long long)blockIdx.x >= tiles) return;
  const unsigned char* img = reinterpret_cast<const unsigned char*>(a.tc_img) + (size_t)op.img * kTcImageBytes;
  const int Ei = reinterpret_cast<const int*>(img)[(32 * ((threadIdx.x >> 5) & 3) + (threadIdx.x & 31)) & 63];
  const double* stage = reinterpret_cast<const double*>(t.a[0]);
  PhaseClock pc{(a.phase && blockIdx.x == 0 && threadIdx.x == 0) ? a.phase : nullptr, 0ull};
  if (pc.acc) pc.t = gtimer();
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    if (pc.acc) pc.acc[14] += 1;
    long long aa = 0, b0 = 0, sn, sj;
    const double2* base;
    if (mode) {
      aa = tile / (nb / TC_N);
      b0 = (tile % (nb / TC_N)) * TC_N;
      base = in + aa * 64 * nb + b0;
      sn = 1;
      sj = nb;
    } else {
      b0 = tile * TC_N;
      base = in + b0 * 64;
      sn = 64;
      sj = 1;
    }
    tc_b_exponents(t, base, sn, sj);
    pc.mark(10);
    // double-buffered chunks: the bulk copy and the slicing of chunk q + 1 overlap the
    // MMAs of chunk q
    if (threadIdx.x == 0) {
      tc::fence_proxy_async_all();
      tc::mbar_expect_tx(&t.lbar[0], (uint32_t)TC_A_CHUNK_BYTES);
      tc::bulk_g2s(t.a[0], img + TC_IMG_HDR, (uint32_t)TC_A_CHUNK_BYTES, &t.lbar[0]);
    }
    tc_stage_b(t, 0, base, sn, sj, 0);
    bool ok = true;
    for (int q = 0; q < TC_CHUNKS; ++q) {
      const int bi = q & 1, nbi = bi ^ 1;
      ok = tc_wait(&t.lbar[bi], t.lph[bi]) && ok;
      tc::fence_proxy_async();
      tc::fence_before();
      __syncthreads();
      tc::fence_after();
      if (threadIdx.x == 0) tc_issue_chunk(t, q, bi);
      __syncwarp();
      if (q + 1 < TC_CHUNKS) {
        if (q >= 1) ok = tc_wait(&t.mbar[nbi], t.mph[nbi]) && ok;  // chunk q - 1 has released buffer nbi
        tc::fence_after();
        if (threadIdx.x == 0) {
          tc::fence_proxy_async_all();
          tc::mbar_expect_tx(&t.lbar[nbi], (uint32_t)TC_A_CHUNK_BYTES);
          tc::bulk_g2s(t.a[nbi], img + TC_IMG_HDR + (size_t)(q + 1) * TC_A_CHUNK_BYTES, (uint32_t)TC_A_CHUNK_BYTES,
                       &t.lbar[nbi]);
        }
        tc_stage_b(t, nbi, base, sn, sj, q + 1);
      }
    }
    // chunks 2 and 3 (buffers 0 and 1) complete
    ok = tc_wait(&t.mbar[0], t.mph[0]) && ok;
    ok = tc_wait(&t.mbar[1], t.mph[1]) && ok;
    tc::fence_after();
    if (!ok && threadIdx.x == 0) atomicOr(a.err, tc::kErrMmaTimeout);
    pc.mark(11);
    tc_drain_to_stage(t, Ei, pc);
    pc.mark(12);
    // stage -> out: element (i, n) = (stage[i][n], stage[64 + i][n]); 64 N / 256 elements
    // per thread in batches of 4 so that the loads of the accumulated outputs overlap
    for (int r0 = 0; r0 < 64 * TC_N / 256; r0 += 4) {
      double2* dst[4];
      double2 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int task = threadIdx.x + 256 * (r0 + u);
        int i, n;
        if (mode) {
          n = task % TC_N;
          i = task / TC_N;
          dst[u] = out + aa * 64 * nb + (long long)i * nb + b0 + n;
        } else {
          i = task & 63;
          n = task >> 6;
          dst[u] = out + (b0 + n) * 64 + i;
        }
        v[u] = make_double2(stage[i * TC_STAGE_LD + n], stage[(64 + i) * TC_STAGE_LD + n]);
      }
      if (acc) {
        double2 o[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) o[u] = *dst[u];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = cadd(v[u], o[u]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) *dst[u] = v[u];
    }
    // the next tile's bulk copies (async proxy) overwrite the stage just read
    tc::fence_proxy_async_all();
    __syncthreads();
    pc.mark(13);
  }
}

__device__ void run_program(const ExpmArgs& a, const double2* x, TcState* t) {
  for (int k = 0; k < a.nops; ++k) {
    const MvOp& op = a.prog[k];
    if (op.barrier_before) grid_barrier(a.bar, a.err);
    if (op.tc && t) run_op_tc(a, op, x, *t);
    else run_op(a, op, x);
  }
  if (a.tail_barrier) grid_barrier(a.bar, a.err);
}

// ---- reductions: partials [gridDim][nq] (complex), reduced by every CTA in block order
__device__ void store_partials(Red& sm, int nq, double2* part) {
  __syncthreads();
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = cadd(s, sm.w[w][q]);
    part[(long long)blockIdx.x * nq + q] = s;
  }
  __syncthreads();
}
// every CTA: out[q] = sum_b part[b][q], threads over (q, b-slices)
__device__ void reduce_partials(const double2* part, int nq, double2* out, Red& sm) {
  const int G = gridDim.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // warp w handles q = w, w+8, ...; lanes stride over b
  for (int q = w; q < nq; q += (int)(blockDim.x >> 5)) {
    double2 s = make_double2(0.0, 0.0);
    for (int b = lane; b < G; b += 32) s = cadd(s, part[(long long)b * nq + q]);
    s = warp_sum2(s);
    if (lane == 0) out[q] = s;
  }
  __syncthreads();
}

// sums over the whole launch of the nq per-warp values in sm.w into out (every CTA): for one
// CTA straight from shared memory (the same order as the two-pass form, which adds only
// zeros past the first partial), else through the partials and a grid barrier
__device__ void launch_sum(const ExpmArgs& a, Red& sm, int nq, double2* part, double2* out) {
  if (gridDim.x == 1) {
    __syncthreads();
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      double2 s = make_double2(0.0, 0.0);
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = cadd(s, sm.w[w][q]);
      out[q] = s;
    }
    __syncthreads();
    return;
  }
  store_partials(sm, nq, part);
  grid_barrier(a.bar, a.err);
  reduce_partials(part, nq, out, sm);
}

// The small exponential of the step control, F = exp(zc * Haug) e1, by one warp.
// Haug is the Lanczos tridiagonal (d on the diagonal, e[i] coupling rows i-1 and i) of
// size mb, bordered when aug is set by row mb = betm at column mb-1 and row mb+1 = 1 at
// column mb (Sidje's augmented matrix, whose rows mb and mb+1 of exp(zc Haug) e1 are
// betm zc e_mb^T phi1(zc T) e1 and betm zc^2 e_mb^T phi2(zc T) e1, the two terms of the
// error estimate).  Evaluated as (sum_{k<=K} (zc Haug / s)^k / k!)^s e1 with s the
// fewest segments of norm r = ||zc Haug / s||_inf <= 4 and K the fewest terms whose
// remainder r^(K+1) e^r / (K+1)! stays below 2^-56 (kTaylorK); every row is one lane, so
// the dependent chain per term is a handful of FP64 operations (FP64 latency and the
// FP64 issue rate of one warp, not throughput, bound this phase on GB300).  When zc is
// real or imaginary (the usual case: coefficient -i and a real time step), the first
// segment, which starts from the real e1, runs in real arithmetic: term k is u^k w_k with
// u in {1, -1, i, -i} and the real recurrence w_k = (|zc| / (s k)) Haug w_{k-1}.
struct CtlSmem {
  double d[EQ], e[EQ + 1];
  double2 x[EQ + 2];
  double2 t[2][EQ + 2];
  double w[2][EQ + 2];
};
constexpr size_t kCtlBytes = (sizeof(CtlSmem) + 255) / 256 * 256;  // where resident vectors start
constexpr int kMaxScaling = 4096;   // ||zc Haug||_inf above this fails the step (error bit 4)
constexpr int kMaxTaylor = 34;
__constant__ unsigned char kTaylorK[32] = {10, 12, 14, 15, 16, 17, 18, 19, 19, 20, 21, 22, 23, 23, 24, 25,
                                           25, 26, 26, 27, 28, 28, 29, 30, 30, 31, 31, 32, 32, 33, 34, 34};
__constant__ double kInvK[kMaxTaylor + 1] = {
    0.0,       1.0,       1.0 / 2,   1.0 / 3,   1.0 / 4,   1.0 / 5,   1.0 / 6,   1.0 / 7,   1.0 / 8,
    1.0 / 9,   1.0 / 10,  1.0 / 11,  1.0 / 12,  1.0 / 13,  1.0 / 14,  1.0 / 15,  1.0 / 16,  1.0 / 17,
    1.0 / 18,  1.0 / 19,  1.0 / 20,  1.0 / 21,  1.0 / 22,  1.0 / 23,  1.0 / 24,  1.0 / 25,  1.0 / 26,
    1.0 / 27,  1.0 / 28,  1.0 / 29,  1.0 / 30,  1.0 / 31,  1.0 / 32,  1.0 / 33,  1.0 / 34};

// row i of Haug applied to a real vector t
__device__ __forceinline__ double haug_row(int i, int mb, double betm, const double* d, const double* e,
                                           const double* t) {
  if (i < mb) {
    double u = d[i] * t[i];
    if (i > 0) u = fma(e[i], t[i - 1], u);
    if (i + 1 < mb) u = fma(e[i + 1], t[i + 1], u);
    return u;
  }
  return (i == mb) ? betm * t[mb - 1] : t[mb];
}

__device__ bool warp_expm_e1(int mb, bool aug, double betm, double2 zc, CtlSmem& S) {
  const int lane = threadIdx.x & 31;
  const int mx = mb + (aug ? 2 : 0);
  if (mx <= 32 && (zc.x == 0.0 || zc.y == 0.0)) {
    // The usual case, one segment (||zc Haug||_inf <= 4) of real arithmetic, in registers:
    // lane i holds row i of Haug as (diagonal, coupling to row i-1, coupling to row i+1)
    // and the current term; the neighbours' terms come by shuffles and the coefficients
    // ck d_i, ck e_i, ck e_{i+1} are formed off the chain, so one Taylor term costs three
    // dependent FP64 operations.  The row-sum maximum is taken on the bit patterns (the
    // sums are non-negative) and |zc| without a hypot.
    double di = 0.0, em = 0.0, ep = 0.0, rs = 0.0;
    if (lane < mb) {
      di = S.d[lane];
      em = lane > 0 ? S.e[lane] : 0.0;
      ep = lane + 1 < mb ? S.e[lane + 1] : 0.0;
      rs = fabs(di) + fabs(em) + fabs(ep);
    } else if (lane == mb && aug) {
      em = betm;
      rs = fabs(betm);
    } else if (lane == mb + 1 && aug) {
      em = 1.0;
      rs = 1.0;
    }
    long long rb = __double_as_longlong(rs);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long t = __shfl_xor_sync(0xffffffffu, rb, o);
      rb = t > rb ? t : rb;
    }
    const bool real_z = (zc.y == 0.0), imag_z = (zc.x == 0.0);
    const double az = real_z ? fabs(zc.x) : fabs(zc.y);
    const double nrm = __longlong_as_double(rb) * az;
    if (nrm <= 4.0) {
      int kb = (int)ceil(nrm * 8.0) - 1;
      kb = kb < 0 ? 0 : (kb > 31 ? 31 : kb);
      const int K = kTaylorK[kb];
      const double sg = real_z ? (zc.x < 0.0 ? -1.0 : 1.0) : (zc.y < 0.0 ? -1.0 : 1.0);
      double t = lane == 0 ? 1.0 : 0.0, x0 = t, x1 = 0.0;
      for (int k = 1; k <= K; ++k) {
        const double ck = az * kInvK[k];
        const double cd = ck * di, ce = ck * em, cp = ck * ep;
        const double tm = __shfl_up_sync(0xffffffffu, t, 1);
        const double tp = __shfl_down_sync(0xffffffffu, t, 1);
        const double tn = fma(cp, tp, fma(ce, tm, cd * t));
        // u^k: real_z: sg^k; imag_z: sg^k i^k
        const bool odd = (k & 1) != 0;
        double sk = odd ? sg : 1.0;
        if (imag_z && (k & 3) >= 2) sk = -sk;
        if (imag_z && odd) x1 = fma(sk, tn, x1);
        else x0 = fma(sk, tn, x0);
        t = tn;
      }
      if (lane < mx) S.x[lane] = make_double2(x0, x1);
      __syncwarp();
      return true;
    }
  }
  double rn = 0.0;
  for (int i = lane; i < mx; i += 32) {
    double r;
    if (i < mb) r = fabs(S.d[i]) + (i > 0 ? fabs(S.e[i]) : 0.0) + (i + 1 < mb ? fabs(S.e[i + 1]) : 0.0);
    else if (i == mb) r = fabs(betm);
    else r = 1.0;
    rn = fmax(rn, r);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rn = fmax(rn, __shfl_xor_sync(0xffffffffu, rn, o));
  const double az = hypot(zc.x, zc.y);
  const double nrm = rn * az;
  if (!(nrm <= (double)kMaxScaling)) return false;
  const int s = nrm > 4.0 ? (int)ceil(nrm * 0.25) : 1;
  const double inv_s = 1.0 / (double)s;
  int kb = (int)ceil(nrm * inv_s * 8.0) - 1;
  kb = kb < 0 ? 0 : (kb > 31 ? 31 : kb);
  const int K = kTaylorK[kb];
  for (int i = lane; i < mx; i += 32) S.x[i] = make_double2(i == 0 ? 1.0 : 0.0, 0.0);
  __syncwarp();
  int rep = 0;
  const bool real_z = (zc.y == 0.0), imag_z = (zc.x == 0.0);
  if (real_z || imag_z) {
    // zc = |zc| u: real_z: u = sign(zc.x); imag_z: u = sign(zc.y) i
    const double sg = real_z ? (zc.x < 0.0 ? -1.0 : 1.0) : (zc.y < 0.0 ? -1.0 : 1.0);
    const double a = az * inv_s;
    for (int i = lane; i < mx; i += 32) S.w[0][i] = (i == 0) ? 1.0 : 0.0;
    __syncwarp();
    double* xs = reinterpret_cast<double*>(S.x);
    int cur = 0;
    for (int k = 1; k <= K; ++k) {
      const double ck = a * kInvK[k];
      // u^k: real_z: sg^k (real part); imag_z: sg^k i^k
      const bool odd = (k & 1) != 0;
      double sk = odd ? sg : 1.0;
      int comp = 0;
      if (imag_z) {
        comp = odd ? 1 : 0;
        if ((k & 3) >= 2) sk = -sk;
      }
      const double* tc = S.w[cur];
      for (int i = lane; i < mx; i += 32) {
        const double v = ck * haug_row(i, mb, betm, S.d, S.e, tc);
        S.w[cur ^ 1][i] = v;
        xs[2 * i + comp] = fma(sk, v, xs[2 * i + comp]);
      }
      __syncwarp();
      cur ^= 1;
    }
    rep = 1;
  }
  for (; rep < s; ++rep) {
    for (int i = lane; i < mx; i += 32) S.t[0][i] = S.x[i];
    __syncwarp();
    int cur = 0;
    for (int k = 1; k <= K; ++k) {
      const double2 ck = cscale(inv_s * kInvK[k], zc);
      const double2* tc = S.t[cur];
      for (int i = lane; i < mx; i += 32) {
        double2 u;
        if (i < mb) {
          u = cscale(S.d[i], tc[i]);
          if (i > 0) u = make_double2(fma(S.e[i], tc[i - 1].x, u.x), fma(S.e[i], tc[i - 1].y, u.y));
          if (i + 1 < mb) u = make_double2(fma(S.e[i + 1], tc[i + 1].x, u.x), fma(S.e[i + 1], tc[i + 1].y, u.y));
        } else if (i == mb) {
          u = cscale(betm, tc[mb - 1]);
        } else {
          u = tc[mb];
        }
        const double2 v = cmul(ck, u);
        S.t[cur ^ 1][i] = v;
        S.x[i] = cadd(S.x[i], v);
      }
      __syncwarp();
      cur ^= 1;
    }
  }
  return true;
}

// The residual stop of a Lanczos recurrence, by warp 0 of block 0 after step jj - 1: ends
// the recurrence at dimension jj (as an exact breakdown does) when
// beta_0 beta_jj |e_{jj-1}^T exp(c tau T_jj) e_1| <= tol for the remaining interval tau.
// Kept out of line so that the registers of the Lanczos loop do not grow.
// The final test compares squares unless they lie within 1e-12 of the threshold, where it
// falls back to the product with the modulus (a hypot costs about 700 cycles of one warp).
__device__ __noinline__ void residual_stop(KrylovCtl* ctl, int jj, int m, double beta, CtlSmem& S) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < jj; i += 32) {
    S.d[i] = ctl->alpha[i];
    S.e[i] = ctl->bet[i];
  }
  __syncwarp();
  const double rest = ctl->t_out - ctl->t_now;
  const double2 zc = cscale(ctl->sgn * rest, make_double2(ctl->cf_re, ctl->cf_im));
  const bool ok = warp_expm_e1(jj, false, 0.0, zc, S);
  if (lane == 0 && ok && ctl->mb == m) {
    const double2 last = S.x[jj - 1];
    const double f = ctl->beta * beta, tol = ctl->tol;
    const double l2 = f * f * fma(last.x, last.x, last.y * last.y), t2 = tol * tol;
    bool stop;
    if (l2 > 1e-290 && l2 < 1e290 && t2 > 1e-290 && t2 < 1e290 && fabs(l2 - t2) > 1e-12 * t2)
      stop = l2 < t2;
    else
      stop = f * hypot(last.x, last.y) <= tol;
    if (stop) {
      ctl->mb = jj;
      ctl->k1 = 0;
    }
  }
  __syncwarp();
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
    S.e[i] = ctl->bet[i];
  }
  __syncwarp();
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
  const double betm = ctl->bet[mb];
  int ireject = 0;
  for (;;) {
    const double t_step = s_tstep;
    const double2 zc = cscale(ctl->sgn * t_step, cf);
    const bool ok = warp_expm_e1(mb, k1 != 0, betm, zc, S);
    if (!ok) {
      if (lane == 0) {
        ctl->err |= 4;
        ctl->done = 1;
      }
      return;
    }
    if (lane == 0) {
      double err_loc, xm = 1.0 / m;
      int accept = 0;
      if (k1 == 0) {
        err_loc = 1e-14;
        accept = 1;
      } else {
        double p1 = hypot(S.x[mb].x, S.x[mb].y) * beta, p2 = hypot(S.x[mb + 1].x, S.x[mb + 1].y) * beta * avnorm;
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
  const double t_step = s_tstep, err_loc = s_err, xm = s_xm;
  const bool good = !s_fail && isfinite(t_step) && t_step > 0.0 && isfinite(err_loc);
  if (good) {
    // the combination coefficients, one per lane
    const int mx = mb + (k1 > 1 ? k1 - 1 : 0);
    for (int q = lane; q < 72; q += 32) {
      const double2 c = (q < mx) ? cscale(beta, S.x[q]) : make_double2(0.0, 0.0);
      ctl->coef[2 * q] = c.x;
      ctl->coef[2 * q + 1] = c.y;
    }
  }
  if (lane == 0) {
    if (s_fail) {
      ctl->err |= 1;
      ctl->done = 1;
    } else if (!good) {
      ctl->err |= 8;
      ctl->done = 1;
    } else {
      const double t_now = ctl->t_now + t_step;
      ctl->t_now = t_now;
      // the next sub-step's size; none follows the last one
      if (k1 != 0 && !(t_now >= ctl->t_out)) {
        double tn = gamma * t_step * pow(t_step * tol / fmax(err_loc, 1e-300), xm);
        double sc = pow(10.0, floor(log10(tn)) - 1.0);
        ctl->t_new = ceil(tn / sc) * sc;
        if (!isfinite(ctl->t_new) || !(ctl->t_new > 0.0)) ctl->t_new = t_step;
      }
      ctl->napps += mb + (k1 != 0 ? 1 : 0);
      ctl->substeps += 1;
      if (t_now >= ctl->t_out) ctl->done = 1;
    }
  }
  __syncwarp();
}

// SV: the one-CTA form with the vectors resident in shared memory (ExpmArgs::smem_vecs; no
// tensor-core ops), a separate instantiation so that the general form keeps its vector
// pointers in the parameter space
template <bool SV>
__global__ void __launch_bounds__(ET, 2) k_expm_coop(ExpmArgs a_in) {
  __shared__ Red sm;
  __shared__ double2 red[EQ];
  __shared__ int s_done, s_mb;
  __shared__ __align__(8) uint64_t s_mbar[2];
  __shared__ __align__(8) uint64_t s_lbar[2];
  __shared__ uint32_t s_tmem;
  extern __shared__ __align__(1024) unsigned char dsm[];
  __shared__ MvOp s_op1;
  // the controller's scratch and the tensor-core operands share the dynamic buffer: they
  // are used in different phases
  CtlSmem& cs = *reinterpret_cast<CtlSmem*>(dsm);
  grid_barrier_begin(a_in.bar);
  // a single contraction passed by value runs from a shared-memory copy
  ExpmArgs a = a_in;
  if (a.prog == nullptr) {
    if (threadIdx.x == 0) s_op1 = a_in.op1;
    __syncthreads();
    a.prog = &s_op1;
  }
  TcState tcs;
  TcState* tcp = nullptr;
  if (!SV && a.mixed) {
    if (threadIdx.x == 0) {
      tc::mbar_init(&s_mbar[0], 1);
      tc::mbar_init(&s_mbar[1], 1);
      tc::mbar_init(&s_lbar[0], 1);
      tc::mbar_init(&s_lbar[1], 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&s_tmem, TC_TMEM_COLS);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    tcs.tmem = s_tmem;
    tcs.mph[0] = tcs.mph[1] = 0;
    tcs.lph[0] = tcs.lph[1] = 0;
    tcs.mbar = s_mbar;
    tcs.lbar = s_lbar;
    tcs.a[0] = dsm;
    tcs.a[1] = dsm + TC_A_CHUNK_BYTES;
    tcs.b[0] = dsm + 2 * TC_A_CHUNK_BYTES;
    tcs.b[1] = dsm + 2 * TC_A_CHUNK_BYTES + TC_B_CHUNK_BYTES;
    tcs.e_n = reinterpret_cast<int*>(dsm + 2 * (TC_A_CHUNK_BYTES + TC_B_CHUNK_BYTES));
    tcp = &tcs;
    build_tc_images(a);
  }
  if (SV) {
    // one CTA, small problem: the basis, p and the temporaries after the controller's
    // scratch, so that the Lanczos passes and the matvec read shared memory, not L2
    double2* b = reinterpret_cast<double2*>(dsm + kCtlBytes);
    a.V = b;
    a.ldv = a.ldt;
    b += (size_t)(a.m + 1) * a.ldt;
    a.p = b;
    a.t1 = b + a.ldt;
    a.t2 = b + 2 * a.ldt;
    a.t3 = b + 3 * a.ldt;
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
  PhaseClock pc{(a.phase && blockIdx.x == 0 && threadIdx.x == 0) ? a.phase : nullptr, 0ull};
  if (pc.acc) {
    pc.t = gtimer();
    pc.acc[9] += 1;
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
      launch_sum(a, sm, 1, pa, red);
    }
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
    if (pc.acc) pc.acc[8] += 1;
    pc.mark(0);
    // ---- Lanczos with full re-orthogonalisation
    double anorm_rows = 0.0;  // breakdown scale: largest row sum of the tridiagonal so far
    for (int j = 0; j < m; ++j) {
      const double2* Vj = a.V + (long long)j * a.ldv;
      grid_barrier(a.bar, a.err);
      // after an exact breakdown the basis is complete: no further vectors
      if (threadIdx.x == 0) s_mb = *(volatile int*)&ctl->mb;
      __syncthreads();
      if (s_mb < m) break;
      run_program(a, Vj, tcp);
      pc.mark(1);
      // partial <V_j, p> over my elements (same element ownership as the last writes of p)
      {
        double2 s = make_double2(0.0, 0.0);
        // two elements per iteration (same summation order): twice the loads in flight
        long long i = tid;
        for (; i + nthreads < n; i += 2 * nthreads) {
          const double2 v0 = Vj[i], p0 = a.p[i], v1 = Vj[i + nthreads], p1 = a.p[i + nthreads];
          s = cadd(s, cmulc(v0, p0));
          s = cadd(s, cmulc(v1, p1));
        }
        if (i < n) s = cadd(s, cmulc(Vj[i], a.p[i]));
        s = warp_sum2(s);
        if (lane == 0) sm.w[warp][0] = s;
        launch_sum(a, sm, 1, pa, red);
      }
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
      pc.mark(2);
      // <V_q, p> for q <= j, four at a time so that the loads and the warp sums of the
      // four overlap
      for (int q0 = 0; q0 <= j; q0 += 4) {
        double2 s[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) s[u] = make_double2(0.0, 0.0);
        for (long long i = tid; i < n; i += nthreads) {
          const double2 pi = a.p[i];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (q0 + u <= j) s[u] = cadd(s[u], cmulc(a.V[(long long)(q0 + u) * a.ldv + i], pi));
        }
        // warp sums of the eight doubles by a transposing butterfly: at offsets 16, 8, 4
        // each lane keeps half of its values and adds the partner's copy of that half, then
        // two plain levels; 9 FP64 additions per lane instead of 40 (one warp's FP64
        // instruction occupies the SM's FP64 pipe for 16 cycles on GB300).  Lane 4 v ends
        // with double v (s[v / 2], real part when v is even).
        {
          double v8[8] = {s[0].x, s[0].y, s[1].x, s[1].y, s[2].x, s[2].y, s[3].x, s[3].y};
          const bool b4 = (lane & 16) != 0, b3 = (lane & 8) != 0, b2 = (lane & 4) != 0;
          double w4[4], w2[2];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const double give = b4 ? v8[k] : v8[k + 4];
            w4[k] = (b4 ? v8[k + 4] : v8[k]) + __shfl_xor_sync(0xffffffffu, give, 16);
          }
#pragma unroll
          for (int k = 0; k < 2; ++k) {
            const double give = b3 ? w4[k] : w4[k + 2];
            w2[k] = (b3 ? w4[k + 2] : w4[k]) + __shfl_xor_sync(0xffffffffu, give, 8);
          }
          double w1 = (b2 ? w2[1] : w2[0]) + __shfl_xor_sync(0xffffffffu, b2 ? w2[0] : w2[1], 4);
          w1 += __shfl_xor_sync(0xffffffffu, w1, 2);
          w1 += __shfl_xor_sync(0xffffffffu, w1, 1);
          const int v = lane >> 2;
          if ((lane & 3) == 0 && q0 + (v >> 1) <= j)
            reinterpret_cast<double*>(&sm.w[warp][q0 + (v >> 1)])[v & 1] = w1;
        }
      }
      if (blockIdx.x == 0 && threadIdx.x == 0) ctl->alpha[j] = alpha;
      if (gridDim.x == 1) {
        launch_sum(a, sm, j + 1, pb, red);
      } else if (gridDim.x >= kSliceReduceGrid) {
        store_partials(sm, j + 1, pb);
        grid_barrier(a.bar, a.err);
        // CTA q < j + 1 reduces coefficient q over all partials (same order as
        // reduce_partials), then everyone reads the j + 1 results: one more barrier instead
        // of every CTA summing (j + 1) x grid partials in FP64
        double2* rq = a.part + (size_t)2 * gridDim.x * EQ;
        if ((int)blockIdx.x <= j && warp == 0) {
          double2 t = make_double2(0.0, 0.0);
          for (int b = lane; b < (int)gridDim.x; b += 32) t = cadd(t, pb[(long long)b * (j + 1) + blockIdx.x]);
          t = warp_sum2(t);
          if (lane == 0) rq[blockIdx.x] = t;
        }
        grid_barrier(a.bar, a.err);
        for (int q = threadIdx.x; q <= j; q += blockDim.x) red[q] = rq[q];
        __syncthreads();
      } else {
        launch_sum(a, sm, j + 1, pb, red);
      }
      pc.mark(3);
      {
        double s = 0.0;
        for (long long i = tid; i < n; i += nthreads) {
          // p -= sum_q c_q V_q in two chains (even and odd q)
          double2 x0 = a.p[i], x1 = make_double2(0.0, 0.0);
          int q = 0;
          for (; q + 2 <= j + 1; q += 2) {
            x0 = csub(x0, cmul(red[q], a.V[(long long)q * a.ldv + i]));
            x1 = csub(x1, cmul(red[q + 1], a.V[(long long)(q + 1) * a.ldv + i]));
          }
          if (q <= j) x0 = csub(x0, cmul(red[q], a.V[(long long)q * a.ldv + i]));
          const double2 x = cadd(x0, x1);
          a.p[i] = x;
          s += x.x * x.x + x.y * x.y;
        }
        s = wsum(s);
        if (lane == 0) sm.w[warp][0] = make_double2(s, 0.0);
        launch_sum(a, sm, 1, pa, red);
      }
      {
        const double beta = sqrt(red[0].x);
        // max over the rows q <= j of |alpha_q| + beta_q + beta_{q+1}: the rows below j were
        // complete at the previous step, row j completes with this beta
        const double vrow = fabs(alpha) + bj + beta;
        const double anorm = vrow > anorm_rows ? vrow : anorm_rows;
        anorm_rows = anorm;
        const int brk = (beta <= 1e-14 * (1.0 + anorm)) ? 1 : 0;
        const double inv = brk ? 0.0 : 1.0 / beta;
        double2* Vn = a.V + (long long)(j + 1) * a.ldv;
        {
          long long i = tid;
          for (; i + nthreads < n; i += 2 * nthreads) {
            const double2 p0 = a.p[i], p1 = a.p[i + nthreads];
            Vn[i] = cscale(inv, p0);
            Vn[i + nthreads] = cscale(inv, p1);
          }
          if (i < n) Vn[i] = cscale(inv, a.p[i]);
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          ctl->bet[j + 1] = brk ? 0.0 : beta;
          if (brk && ctl->mb == m) {
            ctl->mb = j + 1;
            ctl->k1 = 0;
          }
          if (!isfinite(beta)) ctl->err |= 2;
        }
        // residual stop: the (j+1)-dimensional space is enough for the whole remaining
        // interval once beta_0 beta_{j+1} |e_j^T exp(c tau T_{j+1}) e_1| <= tol; it ends the
        // recurrence like an exact breakdown (mb = j + 1, no error-estimate product), so
        // every CTA leaves the loop at the same step after the next grid barrier
        if (a.krylov_stop && blockIdx.x == 0 && warp == 0 && !brk && j + 1 < m)
          residual_stop(ctl, j + 1, m, beta, cs);
        __syncthreads();
      }
      pc.mark(4);
    }
    // ---- ||H V_m|| for the error estimate
    grid_barrier(a.bar, a.err);
    if (threadIdx.x == 0) s_mb = *(volatile int*)&ctl->mb;
    __syncthreads();
    const bool breakdown = s_mb < m;  // no error estimate after an exact breakdown
    if (!breakdown) run_program(a, a.V + (long long)m * a.ldv, tcp);
    {
      double s = 0.0;
      if (!breakdown)
        for (long long i = tid; i < n; i += nthreads) {
          double2 v = a.p[i];
          s += v.x * v.x + v.y * v.y;
        }
      s = wsum(s);
      if (lane == 0) sm.w[warp][0] = make_double2(s, 0.0);
      store_partials(sm, 1, pa);
    }
    grid_barrier(a.bar, a.err);
    pc.mark(5);
    if (blockIdx.x == 0) {
      reduce_partials(pa, 1, red, sm);
      if (threadIdx.x == 0) ctl->avnorm = sqrt(red[0].x);
      __syncthreads();
      if (warp == 0) control(a, cs);
    }
    grid_barrier(a.bar, a.err);
    pc.mark(6);
    // ---- y = sum_q c_q V_q over the basis vectors this sub-step wrote: V_0 .. V_m without a
    // breakdown, V_0 .. V_{mb-1} after one (or after the residual stop).  The vectors past
    // them hold whatever an earlier launch (or nothing) left there, and a zero coefficient
    // times a stale non-finite value would still poison y.
    {
      if (threadIdx.x == 0) {
        const int mbq = *(volatile int*)&ctl->mb, k1q = *(volatile int*)&ctl->k1;
        const int nq = mbq + (k1q > 1 ? k1q - 1 : 0);
        s_mb = nq < 1 ? 1 : (nq > m + 1 ? m + 1 : nq);
      }
      for (int q = threadIdx.x; q <= m; q += blockDim.x)
        red[q] = make_double2(ctl->coef[2 * q], ctl->coef[2 * q + 1]);
      __syncthreads();
      const int nq = s_mb;
      for (long long i = tid; i < n; i += nthreads) {
        double2 s = make_double2(0.0, 0.0);
        for (int q = 0; q < nq; ++q) s = cfma(red[q], a.V[(long long)q * a.ldv + i], s);
        a.y[i] = s;
      }
      __syncthreads();
    }
    pc.mark(7);
  }
  if (!SV && a.mixed) {
    tc::fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
      tc::fence_after();
      tc::tmem_dealloc(tcs.tmem, TC_TMEM_COLS);
    }
  }
  grid_barrier_end(a.bar);
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

size_t expm_smem_vecs_bytes(int m, long long ldt) { return kCtlBytes + (size_t)(m + 5) * (size_t)ldt * sizeof(double2); }

// the opt-in shared memory per block less the kernel's static shared memory (the same for
// every GB300; looked up once)
size_t expm_smem_vecs_max_bytes() {
  static long long v = -1;
  if (v < 0) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, k_expm_coop<true>);
    v = (long long)optin - (long long)fa.sharedSizeBytes;
    if (v < 0) v = 0;
  }
  return (size_t)v;
}

int expm_coop_max_grid(int mixed) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(k_expm_coop<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem(1));
  cudaFuncSetAttribute(k_expm_coop<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)expm_smem_vecs_max_bytes());
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_expm_coop<false>, ET, dyn_smem(mixed));
  return sms * (per < 1 ? 1 : per);
}

// partials of two reductions ([grid][EQ] complex each) and the reduced coefficients
size_t expm_partial_bytes(int max_grid) { return (size_t)(2 * max_grid + 1) * EQ * sizeof(double2); }

cudaError_t expm_coop(const ExpmArgs& a, int grid, cudaStream_t s, int threads) {
  if (threads <= 0 || threads > ET || (threads & 31) || a.mixed) threads = ET;  // tensor-core ops need ET
  ExpmArgs b = a;
  size_t dyn = dyn_smem(a.mixed);
  if (a.smem_vecs) {
    if (grid != 1 || a.mixed || a.apply_only || a.ldt < a.n || expm_smem_vecs_bytes(a.m, a.ldt) > expm_smem_vecs_max_bytes())
      return cudaErrorInvalidValue;
    dyn = expm_smem_vecs_bytes(a.m, a.ldt);
  }
  void* args[] = {&b};
  ++g_launches;
  return cudaLaunchCooperativeKernel(a.smem_vecs ? (const void*)k_expm_coop<true> : (const void*)k_expm_coop<false>,
                                     dim3(grid), dim3(threads), args, dyn, s);
}

}  // namespace ttn
