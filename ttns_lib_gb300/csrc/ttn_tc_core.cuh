// tcgen05 building blocks (sm_100 family): TMEM allocation, shared-memory matrix
// descriptors, TF32 MMA issue/commit, mbarrier waits with a bound, TMEM loads.
//
// Operand layout in shared memory: K-major, no swizzle, in 8-row x 16-byte core
// matrices.  For an operand of R rows (R a multiple of 8) and K tf32 elements per row,
// element (row, k) lives at byte
//     ((k / 4) * (R / 8) + row / 8) * 128 + (row % 8) * 16 + (k % 4) * 4
// so the core matrices adjacent in the row (M/N) dimension are 128 bytes apart (SBO) and
// those adjacent in K are (R / 8) * 128 bytes apart (LBO).  One MMA with K = 8 reads two
// k-groups starting at k-group 2*kk.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace ttn {
namespace tc {

constexpr int kMaxWaitSpins = 1 << 24;   // bounded mbarrier waits
enum : int { kErrMmaTimeout = 1 << 13 };

__host__ __device__ constexpr uint32_t tf32_offset(int row, int k, int R) {
  return (uint32_t)((k / 4) * (R / 8) + row / 8) * 128u + (uint32_t)(row % 8) * 16u + (uint32_t)(k % 4) * 4u;
}

// Instruction descriptor, kind::tf32: D F32, A and B TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor, kind::f16 with BF16 A and B (both K-major), D F32, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// 16-bit operand, K-major, no swizzle: element (row, k) of an R-row operand at byte
//   ((k / 8) * (R / 8) + row / 8) * 128 + (row % 8) * 16 + (k % 8) * 2
// (core matrices of 8 rows x 16 bytes; LBO = (R / 8) * 128, SBO = 128; one MMA, K = 16,
// reads the k-groups 2 kk and 2 kk + 1).
__host__ __device__ constexpr uint32_t b16_offset(int row, int k, int R) {
  return (uint32_t)((k / 8) * (R / 8) + row / 8) * 128u + (uint32_t)(row % 8) * 16u + (uint32_t)(k % 8) * 2u;
}

// Shared-memory matrix descriptor (no swizzle, descriptor version 1).
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm volatile("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// x (double) -> tf32 hi + tf32 lo with x ~ hi + lo (about 22 significant bits)
__device__ __forceinline__ void split_tf32(double x, uint32_t& hi, uint32_t& lo) {
  float xf = (float)x;
  hi = to_tf32(xf);
  float r = (float)(x - (double)__uint_as_float(hi));
  lo = to_tf32(r);
}

// ---- TMEM (one warp executes these)
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_slot)),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ---- MMA issue (single thread)
__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

// ---- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}
// returns false if the wait gave up
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity) {
  const uint32_t a = smem_u32(mbar);
  for (int it = 0; it < kMaxWaitSpins; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// ---- bulk copies global -> shared (TMA, 1-D), completing on an mbarrier
__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes) : "memory");
}
// dst and src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(mbar))
               : "memory");
}
// order this thread's generic-proxy writes (global or shared) before later async-proxy accesses
__device__ __forceinline__ void fence_proxy_async_all() { asm volatile("fence.proxy.async;" ::: "memory"); }

// ---- conversions on the integer pipe (FP64 is slow on this part): f64 -> f32 truncating
// the mantissa, f32 -> f64 exact; magnitudes below the f32 normal range become zero
__device__ __forceinline__ float f64_to_f32_int(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
  uint32_t r;
  if (e <= 0) r = sign;
  else if (e >= 255) r = sign | 0x7F800000u;
  else r = sign | ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7FFFFFu);
  return __uint_as_float(r);
}
__device__ __forceinline__ double f32_to_f64_int(float x) {
  const uint32_t b = __float_as_uint(x);
  const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
  const uint32_t e = (b >> 23) & 0xFF;
  unsigned long long r;
  if (e == 0) r = sign;
  else if (e == 255) r = sign | 0x7FF0000000000000ull | ((unsigned long long)(b & 0x7FFFFFu) << 29);
  else r = sign | ((unsigned long long)(e + 896) << 52) | ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)r);
}
// f32 -> tf32 hi + tf32 lo, hi + lo ~ x to about 22 bits
__device__ __forceinline__ void split_tf32_f(float x, uint32_t& hi, uint32_t& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}

// ---- TMEM -> registers: 8 consecutive fp32 columns, no wait (pair with tmem_wait_ld)
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- TMEM -> registers: 16 consecutive fp32 columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace ttn
