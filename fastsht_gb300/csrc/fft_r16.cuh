// Register-blocked ring DFT passes in df64 (the split-precision form's ring FFTs).
//
// The same transforms as fft_passes.cuh (decimation in frequency, natural order in, bin q of a
// 2^logT-point transform at bit-reverse(q); the inverse as the mirrored decimation in time;
// Bluestein around them; an optional radix-3 pass for 3 * 2^logT sizes), with the power-of-two
// part done as radix-16 passes: each thread loads 16 elements of one butterfly from shared
// memory, transforms them in registers (a 4 x 4 split with the constant factors of
// exp(-2 pi i / 16) between the halves), multiplies by the pass's twiddles and stores once.
// Against radix-4 passes the floating-point work per point is the same (about 30 FP32
// instructions per point and bit) but every element crosses shared memory, loads a twiddle and
// has its address computed half as often, and a transform takes half the barriers.  A
// 2^logT-point transform is floor(logT / 4) radix-16 passes and one twiddle-free radix-2^(logT
// mod 4) pass (radix-16 when logT mod 4 = 0).
//
// Output order: the DIF pass at span S = 16 h stores output k of the butterfly at h *
// bitrev4(k), the place four radix-2 DIF levels would put it, so the whole transform leaves bin
// q at bit-reverse(q) exactly as the radix-4 passes do (the Bluestein filter spectrum, which is
// stored in transform order, and dft_bin() are shared with them).
#pragma once
#include "common.cuh"
#include "df64.cuh"
#include "fft_passes.cuh"

// Twiddles of the radix-16 passes, df64, one table per plan: for each span S = 2^s with
// s = 5..logTmax, at fsht_tw16_off(s), 15 rows k = 1..15 of S/16 entries W_S^(j k),
// W_S = exp(-2 pi i / S), j < S/16 (the threads of a warp read consecutive j).
FSHT_HD long long fsht_tw16_off(int s) { return 15LL * ((1LL << (s - 4)) - 2); }
FSHT_HD long long fsht_tw16_entries(int Tmax) {
  return Tmax >= 32 ? 15LL * (Tmax / 8 - 2) : 0;
}

// Shared-memory position of element i: the low three bits (eight 16-byte elements = one
// 128-byte row) XORed with f(r), r = i >> 3.  f is linear in the bits of r and chosen so that
// every group of eight threads touches eight different 16-byte bank groups in each access the
// passes make: rows of eight consecutive elements (sub-stride h >= 8), the radix-16 butterflies
// with h = 4, 2, 1 (rows 8, 4 and 2 apart), the last radix-8 / 4 / 2 passes, and (the r >> hs
// term, hs = logT - 6) the fold's reads of bins in bit-reversed order.
struct Swz16 {
  int hs;
  __device__ __forceinline__ explicit Swz16(const FshtRingFFT& rf)
      : hs(rf.logT > 10 ? rf.logT - 6 : 4) {}
  __device__ __forceinline__ int operator()(int i) const {
    const int r = i >> 3;
    return i ^ (((r >> 1) ^ (-(r & 1)) ^ (r >> hs)) & 7);
  }
};

namespace r16 {
using namespace fftp;

constexpr double kC8 = 0.92387953251128675613;   // cos(pi / 8)
constexpr double kS8 = 0.38268343236508977173;   // sin(pi / 8)
constexpr double kR2 = 0.70710678118654752440;   // sqrt(1 / 2)
constexpr float kC8h = (float)kC8, kC8l = (float)(kC8 - (double)kC8h);
constexpr float kS8h = (float)kS8, kS8l = (float)(kS8 - (double)kS8h);
constexpr float kR2h = (float)kR2, kR2l = (float)(kR2 - (double)kR2h);

// x k for a real df64 constant k = kh + kl, lazy (the low part not renormalised)
__device__ __forceinline__ void mulk(float xh, float xl, float kh, float kl, float& h, float& l) {
  const float p = __fmul_rn(xh, kh);
  float e = __fmaf_rn(xh, kh, -p);
  e = __fmaf_rn(xh, kl, e);
  e = __fmaf_rn(xl, kh, e);
  h = p;
  l = e;
}

// a (c + i s) for df64 constants c, s (lazy)
__device__ __forceinline__ cdd cmulk(cdd a, float ch, float cl, float sh, float sl) {
  cdd w;
  w.h = make_float2(ch, sh);
  w.l = make_float2(cl, sl);
  return cmul_lz(a, w);
}

// Products with the factors of the eighth roots of unity: a (1 -+ i) sqrt(1/2) (W16^2 and its
// conjugate) and a (-1 -+ i) sqrt(1/2) (W16^6): two additions and two products by the df64
// constant sqrt(1/2), lazy.
template <bool INV>
__device__ __forceinline__ cdd mul_w2(cdd a) {   // W16^2 = (1 - i)/sqrt2; inverse (1 + i)/sqrt2
  float uh, ul, vh, vl;
  if (!INV) {
    dd::add_lazy(a.h.x, a.l.x, a.h.y, a.l.y, uh, ul);     // re + im
    dd::add_lazy(a.h.y, a.l.y, -a.h.x, -a.l.x, vh, vl);   // im - re
  } else {
    dd::add_lazy(a.h.x, a.l.x, -a.h.y, -a.l.y, uh, ul);   // re - im
    dd::add_lazy(a.h.x, a.l.x, a.h.y, a.l.y, vh, vl);     // re + im
  }
  cdd r;
  mulk(uh, ul, kR2h, kR2l, r.h.x, r.l.x);
  mulk(vh, vl, kR2h, kR2l, r.h.y, r.l.y);
  return r;
}
template <bool INV>
__device__ __forceinline__ cdd mul_w6(cdd a) {   // W16^6 = (-1 - i)/sqrt2; inverse (-1 + i)/sqrt2
  float uh, ul, vh, vl;
  if (!INV) {
    dd::add_lazy(a.h.y, a.l.y, -a.h.x, -a.l.x, uh, ul);   // im - re
    dd::add_lazy(-a.h.x, -a.l.x, -a.h.y, -a.l.y, vh, vl); // -(re + im)
  } else {
    dd::add_lazy(-a.h.x, -a.l.x, -a.h.y, -a.l.y, uh, ul); // -(re + im)
    dd::add_lazy(a.h.x, a.l.x, -a.h.y, -a.l.y, vh, vl);   // re - im
  }
  cdd r;
  mulk(uh, ul, kR2h, kR2l, r.h.x, r.l.x);
  mulk(vh, vl, kR2h, kR2l, r.h.y, r.l.y);
  return r;
}
// W16^e for e = 1, 3, 9 (forward: exp(-2 pi i e / 16); inverse: the conjugate)
template <bool INV, int E>
__device__ __forceinline__ cdd mul_wg(cdd a) {
  const float sg = INV ? 1.f : -1.f;
  if (E == 1) return cmulk(a, kC8h, kC8l, sg * kS8h, sg * kS8l);
  if (E == 3) return cmulk(a, kS8h, kS8l, sg * kC8h, sg * kC8l);
  return cmulk(a, -kC8h, -kC8l, -sg * kS8h, -sg * kS8l);   // E == 9: (-cos, +sin) forward
}
template <bool INV>
__device__ __forceinline__ cdd mul_w4(cdd a) {   // -i forward, +i inverse
  return INV ? cmul_pi(a) : cmul_mi(a);
}

// 4-point DFT in place, natural order in and out (lazy, two additions deep)
template <bool INV>
__device__ __forceinline__ void dft4(cdd& a, cdd& b, cdd& c, cdd& d) {
  const cdd apc = ladd(a, c), amc = lsub(a, c), bpd = ladd(b, d), bmd = lsub(b, d);
  const cdd wb = mul_w4<INV>(bmd);   // -i (b - d) forward
  a = ladd(apc, bpd);
  c = lsub(apc, bpd);
  b = ladd(amc, wb);
  d = lsub(amc, wb);
}
// ... with c = d = 0 (zero-padded inputs): X0 = a + b, X1 = a + wb, X2 = a - b, X3 = a - wb,
// wb = -i b forward (+i b inverse)
template <bool INV>
__device__ __forceinline__ void dft4_half_in(cdd& a, cdd& b, cdd& c, cdd& d) {
  const cdd wb = mul_w4<INV>(b);
  c = lsub(a, b);
  d = lsub(a, wb);
  const cdd a0 = a;
  a = ladd(a0, b);
  b = ladd(a0, wb);
}

__device__ __forceinline__ void norm_all(cdd* x, int n) {
#pragma unroll
  for (int i = 0; i < n; ++i) x[i] = fin(x[i]);
}

// 16-point DFT in registers: y[k] = sum_n x[n] W16^(+-n k), natural order in and out; the
// midpoint is renormalised, the outputs are lazy (two additions deep: the caller multiplies
// or renormalises them).  k = k2 + 4 k1, n = n1 + 4 n2:
//   y[k2 + 4 k1] = sum_n1 W4^(n1 k1) W16^(n1 k2) sum_n2 x[n1 + 4 n2] W4^(n2 k2).
// HALF_IN: x[8..15] are zero.  HALF_OUT: only y[0..7] are wanted (k1 < 2).
template <bool INV, bool HALF_IN = false, bool HALF_OUT = false>
__device__ __forceinline__ void dft16(cdd (&x)[16]) {
#pragma unroll
  for (int n1 = 0; n1 < 4; ++n1) {
    if (HALF_IN) dft4_half_in<INV>(x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]);
    else dft4<INV>(x[n1], x[n1 + 4], x[n1 + 8], x[n1 + 12]);
  }
  // x[n1 + 4 k2] now holds the inner sum for (n1, k2): twiddle W16^(n1 k2)
  x[5] = mul_wg<INV, 1>(x[5]);
  x[9] = mul_w2<INV>(x[9]);
  x[13] = mul_wg<INV, 3>(x[13]);
  x[6] = mul_w2<INV>(x[6]);
  x[10] = mul_w4<INV>(x[10]);
  x[14] = mul_w6<INV>(x[14]);
  x[7] = mul_wg<INV, 3>(x[7]);
  x[11] = mul_w6<INV>(x[11]);
  x[15] = mul_wg<INV, 9>(x[15]);
  norm_all(x, 16);
  // outer 4-point DFTs over n1 for each k2: registers 4 k2 + n1 -> y[k2 + 4 k1] in 4 k2 + k1
  cdd y[16];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    cdd a = x[4 * k2], b = x[4 * k2 + 1], c = x[4 * k2 + 2], d = x[4 * k2 + 3];
    if (HALF_OUT) {
      const cdd apc = ladd(a, c), amc = lsub(a, c), bpd = ladd(b, d), bmd = lsub(b, d);
      y[k2] = ladd(apc, bpd);
      y[k2 + 4] = ladd(amc, mul_w4<INV>(bmd));
    } else {
      dft4<INV>(a, b, c, d);
      y[k2] = a;
      y[k2 + 4] = b;
      y[k2 + 8] = c;
      y[k2 + 12] = d;
    }
  }
#pragma unroll
  for (int k = 0; k < 16; ++k)
    if (!HALF_OUT || k < 8) x[k] = y[k];
}

// 8-point DFT (n = n1 + 2 n2, k = k2 + 4 k1): natural order in and out, lazy outputs
template <bool INV>
__device__ __forceinline__ void dft8(cdd (&x)[8]) {
  dft4<INV>(x[0], x[2], x[4], x[6]);
  dft4<INV>(x[1], x[3], x[5], x[7]);
  // x[n1 + 2 k2]: twiddle W8^(n1 k2) = W16^(2 n1 k2)
  x[3] = mul_w2<INV>(x[3]);
  x[5] = mul_w4<INV>(x[5]);
  x[7] = mul_w6<INV>(x[7]);
  norm_all(x, 8);
  cdd y[8];
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    y[k2] = ladd(x[2 * k2], x[2 * k2 + 1]);
    y[k2 + 4] = lsub(x[2 * k2], x[2 * k2 + 1]);
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = y[k];
}

template <int R>
__device__ __forceinline__ int brev(int k) {
  if (R == 2) return k;
  if (R == 4) return ((k & 1) << 1) | (k >> 1);
  if (R == 8) return ((k & 1) << 2) | (k & 2) | (k >> 2);
  return (int)(__brev((unsigned)k) >> 28);
}

// R-point DFT in registers, natural order in and out, renormalised (R = 2, 4, 8, 16)
template <int R, bool INV>
__device__ __forceinline__ void dft_r(cdd (&x)[R]) {
  if constexpr (R == 16) {
    dft16<INV>(x);
    norm_all(x, 16);
  } else if constexpr (R == 8) {
    dft8<INV>(x);
    norm_all(x, 8);
  } else if constexpr (R == 4) {
    dft4<INV>(x[0], x[1], x[2], x[3]);
    norm_all(x, 4);
  } else {
    const cdd a = x[0];
    x[0] = fin(ladd(a, x[1]));
    x[1] = fin(lsub(a, x[1]));
  }
}

// One radix-16 DIF pass at span S = 2^ls (h = S/16 >= 2), twiddles W_S^(j k) after the
// butterfly, output k at h * bitrev4(k).  half_in: the butterflies' upper eight inputs are
// Bluestein's zero padding (the first pass of a padded transform).
template <class Sw>
__device__ __forceinline__ void pass16_dif(cdd* buf, const Sw& S, int logT, int nblk, int ls,
                                           const cdd* __restrict__ tw16, bool half_in) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lh = ls - 4, h = 1 << lh;
  const int nbf = nblk << (logT - 4);
  const cdd* tw = tw16 + fsht_tw16_off(ls);
  for (int idx = tid; idx < nbf; idx += nt) {
    const int j = idx & (h - 1);
    const int i0 = ((idx >> lh) << ls) + j;   // blocks of T are spans too: (blk, group) packed
    cdd x[16];
    if (half_in) {
#pragma unroll
      for (int n = 0; n < 8; ++n) x[n] = buf[S(i0 + n * h)];
      dft16<false, true>(x);
    } else {
#pragma unroll
      for (int n = 0; n < 16; ++n) x[n] = buf[S(i0 + n * h)];
      dft16<false>(x);
    }
    buf[S(i0)] = fin(x[0]);
#pragma unroll
    for (int k = 1; k < 16; ++k)
      buf[S(i0 + h * brev<16>(k))] = fin(lmul(x[k], ldg_cdd(&tw[(k - 1) * h + j])));
  }
}

// The inverse pass (DIT, conjugate twiddles before the butterfly): reads output k of the
// forward pass at h * bitrev4(k), writes x[n] at n * h.  half_out: only x[0..7] are wanted.
template <class Sw>
__device__ __forceinline__ void pass16_dit(cdd* buf, const Sw& S, int logT, int nblk, int ls,
                                           const cdd* __restrict__ tw16, bool half_out) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lh = ls - 4, h = 1 << lh;
  const int nbf = nblk << (logT - 4);
  const cdd* tw = tw16 + fsht_tw16_off(ls);
  for (int idx = tid; idx < nbf; idx += nt) {
    const int j = idx & (h - 1);
    const int i0 = ((idx >> lh) << ls) + j;
    cdd x[16];
    x[0] = buf[S(i0)];
#pragma unroll
    for (int k = 1; k < 16; ++k)
      x[k] = lmulc(buf[S(i0 + h * brev<16>(k))], ldg_cdd(&tw[(k - 1) * h + j]));
    if (half_out) {
      dft16<true, false, true>(x);
#pragma unroll
      for (int n = 0; n < 8; ++n) buf[S(i0 + n * h)] = fin(x[n]);
    } else {
      dft16<true>(x);
#pragma unroll
      for (int n = 0; n < 16; ++n) buf[S(i0 + n * h)] = fin(x[n]);
    }
  }
}

// The twiddle-free pass at span R (h = 1): forward (DIF, output k at bitrev(k)) or inverse
// (DIT, input k from bitrev(k), natural order out).
template <int R, bool INV, class Sw>
__device__ __forceinline__ void pass_last(cdd* buf, const Sw& S, int n_elems) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int idx = tid; idx < n_elems / R; idx += nt) {
    const int i0 = idx * R;
    cdd x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = buf[S(i0 + (INV ? brev<R>(k) : k))];
    dft_r<R, INV>(x);
#pragma unroll
    for (int k = 0; k < R; ++k) buf[S(i0 + (INV ? k : brev<R>(k)))] = x[k];
  }
}

// Bluestein's middle step on each group of R elements in registers: the forward transform's
// twiddle-free last pass, the filter spectrum (transform order) and the inverse's twiddle-free
// first pass.
template <int R, class Sw>
__device__ __forceinline__ void pass_filter(cdd* buf, const Sw& S, int n_elems,
                                            const cdd* __restrict__ bhat) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int idx = tid; idx < n_elems / R; idx += nt) {
    const int i0 = idx * R;
    cdd x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = buf[S(i0 + k)];
    dft_r<R, false>(x);
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = fin(lmul(x[k], ldg_cdd(&bhat[i0 + brev<R>(k)])));
    dft_r<R, true>(x);
#pragma unroll
    for (int k = 0; k < R; ++k) buf[S(i0 + k)] = x[k];
  }
}

}  // namespace r16

// In-place DIF transform of rf.P points (natural order in, transform order out) with radix-16
// passes.  nz: inputs at nz and above are zero (Bluestein), which the first radix-16 pass skips
// when they fill the upper half of every butterfly.  last = false: stop before the
// twiddle-free last pass (Bluestein fuses it with the filter).  All threads call it; it
// synchronises on entry and after every pass.
// GEN = false: the caller guarantees a power-of-two size (no radix-3 pass), and the code for
// the other sizes is left out of the kernel (a smaller kernel misses the instruction cache
// less: the belt segment's largest stall).
template <class Sw, bool GEN = true>
__device__ void fft_dif16(cdd* buf, const FshtRingFFT& rf, const Sw& S, const cdd* tw16,
                          const cdd* tw3, int nz, bool last) {
  using namespace fftp;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int logT = rf.logT, T = 1 << logT;
  const int nblk = GEN && rf.r3 ? 3 : 1;
  __syncthreads();
  if (GEN && rf.r3) {
    const cdd* t3 = tw3 + 2 * (T - 1);
    const bool c_zero = nz <= 2 * T;   // the third input of every butterfly is padding
    for (int j = tid; j < T; j += nt) {
      const cdd a = buf[S(j)], b = buf[S(j + T)];
      const cdd c = c_zero ? cdd_zero() : buf[S(j + 2 * T)];
      const cdd sm = c_zero ? b : ladd(b, c), df = c_zero ? b : lsub(b, c);
      const cdd t = lsub(a, cscale_p2(sm, 0.5f));
      const cdd u = cmul_pi(cscale_dd(df, kSqrt3HalfHi, kSqrt3HalfLo));
      buf[S(j)] = fin(ladd(a, sm));
      buf[S(j + T)] = fin(lmul(lsub(t, u), ldg_cdd(&t3[2 * j])));
      buf[S(j + 2 * T)] = fin(lmul(ladd(t, u), ldg_cdd(&t3[2 * j + 1])));
    }
    __syncthreads();
  }
  const int rem = logT & 3;
  const int lstop = rem ? rem : 4;   // span of the twiddle-free last pass
  for (int ls = logT; ls > lstop; ls -= 4) {
    const bool half_in = GEN && !rf.r3 && ls == logT && nz <= (T >> 1);
    r16::pass16_dif(buf, S, logT, nblk, ls, tw16, half_in);
    __syncthreads();
  }
  if (!last) return;
  const int n_elems = nblk << logT;
  switch (lstop) {
    case 1: r16::pass_last<2, false>(buf, S, n_elems); break;
    case 2: r16::pass_last<4, false>(buf, S, n_elems); break;
    case 3: r16::pass_last<8, false>(buf, S, n_elems); break;
    default: r16::pass_last<16, false>(buf, S, n_elems); break;
  }
  __syncthreads();
}

// The inverse of fft_dif16 without normalisation (P times the inverse DFT): transform order
// in, natural order out.  Only outputs below nout are wanted (Bluestein keeps nd of P).
// first = false: the twiddle-free first pass was fused into the caller's filter step.
template <class Sw>
__device__ void fft_dit16_inv(cdd* buf, const FshtRingFFT& rf, const Sw& S, const cdd* tw16,
                              const cdd* tw3, int nout, bool first) {
  using namespace fftp;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int logT = rf.logT, T = 1 << logT;
  const int nblk = rf.r3 ? 3 : 1;
  const int rem = logT & 3;
  const int lstop = rem ? rem : 4;
  __syncthreads();
  if (first) {
    const int n_elems = nblk << logT;
    switch (lstop) {
      case 1: r16::pass_last<2, true>(buf, S, n_elems); break;
      case 2: r16::pass_last<4, true>(buf, S, n_elems); break;
      case 3: r16::pass_last<8, true>(buf, S, n_elems); break;
      default: r16::pass_last<16, true>(buf, S, n_elems); break;
    }
    __syncthreads();
  }
  for (int ls = lstop + 4; ls <= logT; ls += 4) {
    const bool half_out = !rf.r3 && ls == logT && nout <= (T >> 1);
    r16::pass16_dit(buf, S, logT, nblk, ls, tw16, half_out);
    __syncthreads();
  }
  if (rf.r3) {
    const cdd* t3 = tw3 + 2 * (T - 1);
    const bool two_blocks = nout <= 2 * T;   // the third block is not wanted
    for (int j = tid; j < T; j += nt) {
      const cdd a = buf[S(j)];
      const cdd b = lmulc(buf[S(j + T)], ldg_cdd(&t3[2 * j]));
      const cdd c = lmulc(buf[S(j + 2 * T)], ldg_cdd(&t3[2 * j + 1]));
      const cdd sm = ladd(b, c), df = lsub(b, c);
      buf[S(j)] = fin(ladd(a, sm));
      const cdd t = lsub(a, cscale_p2(sm, 0.5f));
      const cdd u = cmul_pi(cscale_dd(df, kSqrt3HalfHi, kSqrt3HalfLo));
      buf[S(j + T)] = fin(ladd(t, u));
      if (!two_blocks) buf[S(j + 2 * T)] = fin(lsub(t, u));
    }
    __syncthreads();
  }
}

// DFT of rf.nd points in buf[0..nd), forward; bin q lands at buf[S(dft_bin(rf, q))] (as
// ring_dft in fft_passes.cuh, with the radix-16 passes).
// GEN = false: every transform the kernel meets is a power of two (no Bluestein, no radix 3).
template <class Sw, bool GEN = true>
__device__ void ring_dft16(cdd* buf, const FshtRingFFT& rf, const Sw& S, const cdd* tw16,
                           const cdd* tw3, const cdd* __restrict__ chirp,
                           const cdd* __restrict__ bhat) {
  using namespace fftp;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (!GEN || !rf.bluestein) {
    fft_dif16<Sw, GEN>(buf, rf, S, tw16, tw3, rf.P, true);
    return;
  }
  const int n = rf.nd, P = rf.P;
  for (int j = tid; j < P; j += nt) {
    if (j < n) buf[S(j)] = fin(lmul(buf[S(j)], ldg_cdd(&chirp[j])));
    else buf[S(j)] = cdd_zero();
  }
  fft_dif16(buf, rf, S, tw16, tw3, n, false);
  const int rem = rf.logT & 3;
  switch (rem) {
    case 1: r16::pass_filter<2>(buf, S, P, bhat); break;
    case 2: r16::pass_filter<4>(buf, S, P, bhat); break;
    case 3: r16::pass_filter<8>(buf, S, P, bhat); break;
    default: r16::pass_filter<16>(buf, S, P, bhat); break;
  }
  fft_dit16_inv(buf, rf, S, tw16, tw3, n, false);
  for (int j = tid; j < n; j += nt) buf[S(j)] = fin(lmul(buf[S(j)], ldg_cdd(&chirp[j])));
  __syncthreads();
}
