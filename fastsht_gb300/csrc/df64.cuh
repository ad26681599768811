// Double-float ("df64") arithmetic: a real value carried as the unevaluated sum hi + lo of
// two FP32 numbers, |lo| about ulp(hi)/2 or less (about 48 significand bits).
//
// Why: GB300 issues FP32 instructions at 64 times its FP64 rate (128 against 2 lanes per clock
// per SM), so FP64-accurate work that is bound by the FP64 pipe runs several times faster in
// this form even though every operation takes 3-19 FP32 instructions.
//
// Error-free building blocks (Knuth's two_sum, Dekker's fast_two_sum, the exact product
// through fmaf); additions are the "sloppy" double-float sum (error below 2^-46 of the
// operands' magnitudes, not of the result's, which is what an FFT's error bound needs).
// Every operation goes through the _rn intrinsics, which the compiler neither contracts into
// FMAs nor reorders.
#pragma once
#include <cuda_runtime.h>

// complex df64: re = h.x + l.x, im = h.y + l.y; 16 bytes like a double2
struct __align__(16) cdd {
  float2 h;
  float2 l;
};

namespace dd {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
}

// exact when |a| >= |b| (or a = 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// (ah + al) + (bh + bl)
__device__ __forceinline__ void add(float ah, float al, float bh, float bl, float& h, float& l) {
  float s, e;
  two_sum(ah, bh, s, e);
  e = __fadd_rn(e, __fadd_rn(al, bl));
  fast_two_sum(s, e, h, l);
}

// x1 y1 + x2 y2: both high products exact through fmaf, their sum through two_sum, the
// error terms and the four cross products gathered in the low part
__device__ __forceinline__ void dot2(float x1h, float x1l, float y1h, float y1l, float x2h,
                                     float x2l, float y2h, float y2l, float& h, float& l) {
  const float p1 = __fmul_rn(x1h, y1h);
  const float e1 = __fmaf_rn(x1h, y1h, -p1);
  const float p2 = __fmul_rn(x2h, y2h);
  const float e2 = __fmaf_rn(x2h, y2h, -p2);
  float s, e;
  two_sum(p1, p2, s, e);
  float t = __fadd_rn(e1, e2);
  t = __fmaf_rn(x1h, y1l, t);
  t = __fmaf_rn(x1l, y1h, t);
  t = __fmaf_rn(x2h, y2l, t);
  t = __fmaf_rn(x2l, y2h, t);
  fast_two_sum(s, __fadd_rn(e, t), h, l);
}

// x y
__device__ __forceinline__ void mul(float xh, float xl, float yh, float yl, float& h, float& l) {
  const float p = __fmul_rn(xh, yh);
  float e = __fmaf_rn(xh, yh, -p);
  e = __fmaf_rn(xh, yl, e);
  e = __fmaf_rn(xl, yh, e);
  fast_two_sum(p, e, h, l);
}

// Lazy forms: the same sums and products without the final fast_two_sum, so the low part
// is not renormalised (|lo| may reach a few ulp(hi); hi + lo still carries the value to about
// 2^-46 of the operands).  Chains of at most a few lazy operations are renormalised when they
// are stored (norm) or converted to FP64.
__device__ __forceinline__ void add_lazy(float ah, float al, float bh, float bl, float& h,
                                         float& l) {
  float e;
  two_sum(ah, bh, h, e);
  l = __fadd_rn(e, __fadd_rn(al, bl));
}

__device__ __forceinline__ void dot2_lazy(float x1h, float x1l, float y1h, float y1l, float x2h,
                                          float x2l, float y2h, float y2l, float& h, float& l) {
  const float p1 = __fmul_rn(x1h, y1h);
  const float e1 = __fmaf_rn(x1h, y1h, -p1);
  const float p2 = __fmul_rn(x2h, y2h);
  const float e2 = __fmaf_rn(x2h, y2h, -p2);
  float e;
  two_sum(p1, p2, h, e);
  float t = __fadd_rn(e1, e2);
  t = __fmaf_rn(x1h, y1l, t);
  t = __fmaf_rn(x1l, y1h, t);
  t = __fmaf_rn(x2h, y2l, t);
  t = __fmaf_rn(x2l, y2h, t);
  l = __fadd_rn(e, t);
}

}  // namespace dd

__device__ __forceinline__ cdd cadd(cdd a, cdd b) {
  cdd r;
  dd::add(a.h.x, a.l.x, b.h.x, b.l.x, r.h.x, r.l.x);
  dd::add(a.h.y, a.l.y, b.h.y, b.l.y, r.h.y, r.l.y);
  return r;
}
__device__ __forceinline__ cdd csub(cdd a, cdd b) {
  cdd r;
  dd::add(a.h.x, a.l.x, -b.h.x, -b.l.x, r.h.x, r.l.x);
  dd::add(a.h.y, a.l.y, -b.h.y, -b.l.y, r.h.y, r.l.y);
  return r;
}
// a w
__device__ __forceinline__ cdd cmul(cdd a, cdd w) {
  cdd r;
  dd::dot2(a.h.x, a.l.x, w.h.x, w.l.x, -a.h.y, -a.l.y, w.h.y, w.l.y, r.h.x, r.l.x);
  dd::dot2(a.h.x, a.l.x, w.h.y, w.l.y, a.h.y, a.l.y, w.h.x, w.l.x, r.h.y, r.l.y);
  return r;
}
// a conj(w)
__device__ __forceinline__ cdd cmulc(cdd a, cdd w) {
  cdd r;
  dd::dot2(a.h.x, a.l.x, w.h.x, w.l.x, a.h.y, a.l.y, w.h.y, w.l.y, r.h.x, r.l.x);
  dd::dot2(a.h.y, a.l.y, w.h.x, w.l.x, -a.h.x, -a.l.x, w.h.y, w.l.y, r.h.y, r.l.y);
  return r;
}
// lazy complex forms (see dd::add_lazy) and the renormalisation
__device__ __forceinline__ cdd cadd_lz(cdd a, cdd b) {
  cdd r;
  dd::add_lazy(a.h.x, a.l.x, b.h.x, b.l.x, r.h.x, r.l.x);
  dd::add_lazy(a.h.y, a.l.y, b.h.y, b.l.y, r.h.y, r.l.y);
  return r;
}
__device__ __forceinline__ cdd csub_lz(cdd a, cdd b) {
  cdd r;
  dd::add_lazy(a.h.x, a.l.x, -b.h.x, -b.l.x, r.h.x, r.l.x);
  dd::add_lazy(a.h.y, a.l.y, -b.h.y, -b.l.y, r.h.y, r.l.y);
  return r;
}
__device__ __forceinline__ cdd cmul_lz(cdd a, cdd w) {
  cdd r;
  dd::dot2_lazy(a.h.x, a.l.x, w.h.x, w.l.x, -a.h.y, -a.l.y, w.h.y, w.l.y, r.h.x, r.l.x);
  dd::dot2_lazy(a.h.x, a.l.x, w.h.y, w.l.y, a.h.y, a.l.y, w.h.x, w.l.x, r.h.y, r.l.y);
  return r;
}
__device__ __forceinline__ cdd cmulc_lz(cdd a, cdd w) {
  cdd r;
  dd::dot2_lazy(a.h.x, a.l.x, w.h.x, w.l.x, a.h.y, a.l.y, w.h.y, w.l.y, r.h.x, r.l.x);
  dd::dot2_lazy(a.h.y, a.l.y, w.h.x, w.l.x, -a.h.x, -a.l.x, w.h.y, w.l.y, r.h.y, r.l.y);
  return r;
}
__device__ __forceinline__ cdd cnorm(cdd a) {
  cdd r;
  dd::fast_two_sum(a.h.x, a.l.x, r.h.x, r.l.x);
  dd::fast_two_sum(a.h.y, a.l.y, r.h.y, r.l.y);
  return r;
}

__device__ __forceinline__ cdd cconj(cdd a) {
  cdd r;
  r.h = make_float2(a.h.x, -a.h.y);
  r.l = make_float2(a.l.x, -a.l.y);
  return r;
}
// -i a
__device__ __forceinline__ cdd cmul_mi(cdd a) {
  cdd r;
  r.h = make_float2(a.h.y, -a.h.x);
  r.l = make_float2(a.l.y, -a.l.x);
  return r;
}
// i a
__device__ __forceinline__ cdd cmul_pi(cdd a) {
  cdd r;
  r.h = make_float2(-a.h.y, a.h.x);
  r.l = make_float2(-a.l.y, a.l.x);
  return r;
}
// a s for a power of two s (exact)
__device__ __forceinline__ cdd cscale_p2(cdd a, float s) {
  cdd r;
  r.h = make_float2(__fmul_rn(a.h.x, s), __fmul_rn(a.h.y, s));
  r.l = make_float2(__fmul_rn(a.l.x, s), __fmul_rn(a.l.y, s));
  return r;
}
// a k for a real df64 constant k = kh + kl
__device__ __forceinline__ cdd cscale_dd(cdd a, float kh, float kl) {
  cdd r;
  dd::mul(a.h.x, a.l.x, kh, kl, r.h.x, r.l.x);
  dd::mul(a.h.y, a.l.y, kh, kl, r.h.y, r.l.y);
  return r;
}
__device__ __forceinline__ cdd cdd_zero() {
  cdd r;
  r.h = make_float2(0.f, 0.f);
  r.l = make_float2(0.f, 0.f);
  return r;
}
__device__ __forceinline__ cdd ldg_cdd(const cdd* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  cdd r;
  r.h = make_float2(v.x, v.y);
  r.l = make_float2(v.z, v.w);
  return r;
}

// ------------------------------------------------------------------ FP64 <-> df64
// x 2^-sh as df64, by bit manipulation (no FP64 instruction): hi = the top 24 significand bits
// (truncated), lo = the remaining 29 bits rounded to 24.  Callers pick sh from the largest
// exponent of the row they convert, so values whose scaled exponent is below -126 are below
// 2^-126 of that row's largest value and flush to zero; NaN and infinity give NaN.
__device__ __forceinline__ float2 dd_from_double(double x, int sh) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hw = (unsigned)(u >> 32);
  const int E = (int)((hw >> 20) & 0x7ff);
  const unsigned sign = hw & 0x80000000u;
  if (E == 0x7ff) return make_float2(__uint_as_float(0x7fc00000u), 0.f);
  const int eh = E - 1023 - sh;
  if (E == 0 || eh < -126) return make_float2(0.f, 0.f);
  const unsigned mhi = hw & 0xfffffu;                 // significand bits 51..32
  const unsigned lw = (unsigned)u;                    // significand bits 31..0
  const unsigned top23 = (mhi << 3) | (lw >> 29);
  const float hi = __uint_as_float(sign | ((unsigned)(eh + 127) << 23) | top23);
  float lo = 0.f;
  if (eh >= -74) {
    const unsigned r = lw & 0x1fffffffu;              // 29 bits
    const float rlo = __fsub_rn(__uint_as_float(0x4b000000u | (r & 0x7fffffu)), 8388608.f);
    const float rhi = __fsub_rn(__uint_as_float(0x4b000000u | (r >> 23)), 8388608.f);
    const float rf = __fmaf_rn(rhi, 8388608.f, rlo);  // r rounded to 24 bits
    lo = __fmul_rn(rf, __uint_as_float((unsigned)(eh - 52 + 127) << 23));
    lo = __uint_as_float(__float_as_uint(lo) ^ sign);
  }
  return make_float2(hi, lo);
}

// float f 2^sh as a double, by bit manipulation; zero and subnormal f give 0, NaN / infinity NaN
__device__ __forceinline__ double dd_float_to_double(float f, int sh) {
  const unsigned b = __float_as_uint(f);
  const int ef = (int)((b >> 23) & 0xff);
  if (ef == 0xff) return __longlong_as_double(0x7ff8000000000000LL);
  const int E = ef - 127 + 1023 + sh;
  if (ef == 0 || E <= 0) return 0.0;
  if (E >= 0x7ff) return (b & 0x80000000u) ? -__longlong_as_double(0x7ff0000000000000LL)
                                            : __longlong_as_double(0x7ff0000000000000LL);
  const unsigned hw = (b & 0x80000000u) | ((unsigned)E << 20) | ((b & 0x7fffffu) >> 3);
  const unsigned lw = b << 29;
  return __hiloint2double((int)hw, (int)lw);
}

// (h + l) 2^sh in FP64 (one FP64 addition)
__device__ __forceinline__ double dd_to_double(float h, float l, int sh) {
  return dd_float_to_double(h, sh) + dd_float_to_double(l, sh);
}

// dd_float_to_double for |sh| <= 896, where no exponent can leave the FP64 range: the double's
// high word is the float's bits shifted right by three with the exponent rebiased by one
// addition (e896 = (896 + sh) << 20) and the sign put back; zero, subnormal and non-finite f
// take the checked path.
__device__ __forceinline__ double dd_float_to_double_near(float f, int sh, unsigned e896) {
  const unsigned b = __float_as_uint(f);
  if ((((b >> 23) & 0xffu) - 1u) >= 254u) return dd_float_to_double(f, sh);
  const unsigned hw = (((b >> 3) & 0x0fffffffu) + e896) | (b & 0x80000000u);
  return __hiloint2double((int)hw, (int)(b << 29));
}

// dd_to_double for |sh| <= 896 (see dd_float_to_double_near)
__device__ __forceinline__ double dd_to_double_near(float h, float l, int sh, unsigned e896) {
  return dd_float_to_double_near(h, sh, e896) + dd_float_to_double_near(l, sh, e896);
}

// the largest biased FP64 exponent field of x (0 for zero / subnormal)
__device__ __forceinline__ int dd_exp_field(double x) {
  return (int)(((unsigned)(__double_as_longlong(x) >> 32) >> 20) & 0x7ff);
}
