// Thin inline-PTX helpers for Blackwell (sm_103a): mbarriers, bulk async copies,
// tcgen05 (UMMA) descriptors, MMA, commit and TMEM loads.  Every wait is bounded:
// on expiry it raises a CTA-wide abort flag and the caller unwinds.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: returns false (and sets *abort) when the phase does not complete
// within the iteration budget or when another thread already aborted.
constexpr uint32_t kWaitLimit = 1u << 24;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          volatile int* abort) {
  for (uint32_t it = 0; it < kWaitLimit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort) return false;
    if (it > 64) __nanosleep(32);
  }
  *abort = 1;
  return false;
}

// 1-D bulk copy global -> shared, completion signalled on an mbarrier (TMA engine).
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ------------------------------------------------------------------ UMMA
// Shared-memory matrix descriptor, no swizzle, K-major core matrices (8 rows x 16 B):
// lbo = byte stride between core matrices adjacent along K, sbo = along M/N.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;   // descriptor version for tcgen05
  return d;
}
// Instruction descriptor, kind::f16: BF16 x BF16 -> F32, both operands K-major.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive on bar when every previously issued tcgen05.mma of this thread completes.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// 32 lanes x 32 bit, 16 consecutive columns per thread.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                 "=r"(v[6]), "=r"(v[7])
               : "r"(taddr)
               : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ------------------------------------------------------------------ slicing
// Operands are cut into four balanced base-256 digits against a power-of-two scale 2^E
// (|v| < 2^E):  v 2^(6-E) = d0 + d1 2^-8 + d2 2^-16 + d3 2^-24 + r,  |r| < 1.5 2^-25,
// |d0| <= 64, |d1..3| <= 128.  Each digit is an integer that BF16 holds exactly, so the
// products of two digits are exact integers; the digit functions below work on the FP32 pipe
// and with 32-bit integer operations (no FP64 instruction).

// The BF16 digit h times 2^-8 (exact: only the exponent moves; digits are >= 1 in
// magnitude, so the result stays normal).
__device__ __forceinline__ uint16_t bf16_scale_2m8(uint16_t h) {
  return (h & 0x7FFF) ? (uint16_t)(h - (8u << 7)) : h;
}
// A digit function returns true when its value does not fit the scale (|v| > 2^E beyond
// rounding, or v is not finite): the digits are then zero and the caller raises the plan's
// error word (kErrRange), so a wrong result never passes silently.
constexpr int kErrTimeout = 1;   // error-word bit: a bounded wait expired
constexpr int kErrRange = 2;     // error-word bit: a value fell outside its digit scale

// f 2^k for an FP32 f, by moving its exponent field (no FP64 and no exp2f range limit): values
// that would leave FP32's normal range below give 0 (far under every digit), above give
// infinity (reported out of range by the caller).
__device__ __forceinline__ float scale_pow2(float f, int k) {
  const unsigned b = __float_as_uint(f);
  const int eb = (int)((b >> 23) & 0xFF);
  if (eb == 0) return 0.f;
  const int ne = eb + k;
  if (ne <= 0) return 0.f;
  if (ne >= 255) return __uint_as_float((b & 0x80000000u) | 0x7F800000u);
  return __uint_as_float((b & 0x807FFFFFu) | ((unsigned)ne << 23));
}

// BF16 bits of a float that holds an integer of magnitude <= 256 (its low 16 bits are zero).
__device__ __forceinline__ uint16_t bf16_of_small_int_float(float d) {
  return (uint16_t)(__float_as_uint(d) >> 16);
}

// Round to the nearest integer, ties to even, on the FP32 add pipe (|x| <= 2^22): adding and
// subtracting 1.5 2^23 leaves no fraction bits.
__device__ __forceinline__ float rint_small(float x) {
  return __fsub_rn(__fadd_rn(x, 0x1.8p23f), 0x1.8p23f);
}

// The digits of w = wh + wl (|wl| <= ulp(wh), |w| <= 64.5) on the FP32 pipe: d0 = rint(wh),
// r = (wh - d0) + wl (the one rounding, below 2^-26), d_{j+1} = rint(256 r_j),
// r_{j+1} = 256 r_j - d_{j+1} (exact).  |d0| <= 64, |d1..3| <= 128 (digits may differ in sign:
// every product stays an exact integer and the level bounds of the contraction hold),
// residual below 1.5 2^-25; the BF16 digits are the high halves of the FP32 digits.
__device__ __forceinline__ void digits_of_pair(float wh, float wl, uint16_t (&s)[4]) {
  const float d0 = rint_small(wh);
  float t = __fmul_rn(__fadd_rn(__fsub_rn(wh, d0), wl), 256.f);
  const float d1 = rint_small(t);
  t = __fmul_rn(__fsub_rn(t, d1), 256.f);
  const float d2 = rint_small(t);
  t = __fmul_rn(__fsub_rn(t, d2), 256.f);
  const float d3 = rint_small(t);
  s[0] = bf16_of_small_int_float(d0);
  s[1] = bf16_of_small_int_float(d1);
  s[2] = bf16_of_small_int_float(d2);
  s[3] = bf16_of_small_int_float(d3);
}

// Four balanced base-256 digits of a df64 value hi + lo (|lo| <= ulp(hi)) against 2^E:
// w = (hi + lo) 2^(6 - E) by exponent moves (exact), then digits_of_pair.  Non-finite hi or
// |hi + lo| > 2^E (beyond rounding) report out of range; the digits are then zero.
__device__ __forceinline__ bool digits4_df(float hi, float lo, int E, uint16_t (&s)[4]) {
  const int k = 6 - E;
  const float wh = scale_pow2(hi, k), wl = scale_pow2(lo, k);
  if (!(fabsf(wh) <= 64.5f)) {                       // also catches infinity and NaN
    s[0] = s[1] = s[2] = s[3] = 0;
    return true;
  }
  digits_of_pair(wh, wl, s);
  return false;
}

// The digits of an FP64 value with FP32 and 32-bit integer operations only: w = v 2^(6 - E) is
// cut from v's bits into an FP32 pair (the top 24 significand bits, then the next 24 of the
// remaining 29, truncated: below 2^-47 of w), then digits_of_pair.  Zero and subnormal v give
// zero digits (below every digit of any scale the kernels use); |v| > 2^E (beyond rounding) or
// a non-finite v report out of range with zero digits.
__device__ __forceinline__ bool digits4_f(double v, int E, uint16_t (&s)[4]) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const int eb = (int)((hw >> 20) & 0x7FF);
  const int ew = eb - 1023 + 6 - E;                   // exponent of w
  s[0] = s[1] = s[2] = s[3] = 0;
  if (eb == 0x7FF || (eb != 0 && ew > 6)) return true;
  if (eb == 0 || ew < -40) return false;              // |w| < 2^-39: all digits zero
  const unsigned sign = hw & 0x80000000u;
  const float wh =
      __uint_as_float(sign | ((unsigned)(ew + 127) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
  const unsigned r = lw & 0x1FFFFFFFu;
  float wl = 0.f;
  if (r) {
    const int p = 31 - __clz(r);                      // leading bit of the remainder
    const unsigned mr = p >= 23 ? (r >> (p - 23)) : (r << (23 - p));
    wl = __uint_as_float(sign | ((unsigned)(ew - 52 + p + 127) << 23) | (mr & 0x7FFFFFu));
  }
  if (!(fabsf(wh) <= 64.5f)) return true;
  digits_of_pair(wh, wl, s);
  return false;
}

}  // namespace tc
