// Shared-memory ring DFT passes, written once for two element types:
//   double2 - FP64 complex (the plain path; every FP64 operation of the earlier FP64-only
//             kernels is kept, including the FMA-folded inverse butterflies)
//   cdd     - df64 complex (df64.cuh), FP64-class accuracy on the FP32 pipe
// Both are 16 bytes, so shared-memory layouts and sizes do not depend on the type.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "df64.cuh"

// Twiddle tables of one element type, packed per pass (fsht_tw_entries in common.cuh): r4 the
// radix-4 triples of each span, r3 the radix-3 pairs of each 3*2^k size.
template <class E>
struct FftTwT {
  const E* r4;
  const E* r3;
};
using FftTw = FftTwT<double2>;

namespace fftp {

constexpr double kSqrt3Half = 0.86602540378443864676;
constexpr float kSqrt3HalfHi = (float)kSqrt3Half;
constexpr float kSqrt3HalfLo = (float)(kSqrt3Half - (double)kSqrt3HalfHi);

__device__ __forceinline__ double2 ldg_e(const double2* p) { return __ldg(p); }
__device__ __forceinline__ cdd ldg_e(const cdd* p) { return ldg_cdd(p); }
__device__ __forceinline__ double2 cmulc(double2 a, double2 w) { return cmul(a, cconj(w)); }
__device__ __forceinline__ double2 cmul_mi(double2 a) { return make_double2(a.y, -a.x); }
// Operations inside one butterfly: exact FP64 for double2; lazy df64 (no renormalisation,
// at most four in a chain) for cdd, renormalised once when the butterfly stores (fin).
__device__ __forceinline__ double2 ladd(double2 a, double2 b) { return cadd(a, b); }
__device__ __forceinline__ double2 lsub(double2 a, double2 b) { return csub(a, b); }
__device__ __forceinline__ double2 lmul(double2 a, double2 w) { return cmul(a, w); }
__device__ __forceinline__ double2 lmulc(double2 a, double2 w) { return cmulc(a, w); }
__device__ __forceinline__ double2 fin(double2 a) { return a; }
__device__ __forceinline__ cdd ladd(cdd a, cdd b) { return cadd_lz(a, b); }
__device__ __forceinline__ cdd lsub(cdd a, cdd b) { return csub_lz(a, b); }
__device__ __forceinline__ cdd lmul(cdd a, cdd w) { return cmul_lz(a, w); }
__device__ __forceinline__ cdd lmulc(cdd a, cdd w) { return cmulc_lz(a, w); }
__device__ __forceinline__ cdd fin(cdd a) { return cnorm(a); }
template <class E> __device__ __forceinline__ E zero_e();
template <> __device__ __forceinline__ double2 zero_e<double2>() { return make_double2(0.0, 0.0); }
template <> __device__ __forceinline__ cdd zero_e<cdd>() { return cdd_zero(); }

}  // namespace fftp

// Shared-memory position of transform element i of a ring's buffer: the low three bits (eight
// 16-byte elements = one 128-byte bank row) are XORed with a function of the row r = i >> 3,
// so every group of eight threads of a warp touches eight different 16-byte bank groups:
//   r ^ ((r & 2) << 1)  - the strided passes with spans 4 and 16 (rows r, r + 2 and
//                         r .. r + 3 of one group of eight rows map to disjoint halves),
//   r >> hs             - the top three bits of a 2^logT-point index, so bins read in
//                         bit-reversed order (the fold after a power-of-two transform) spread
//                         too (hs = logT - 6, at least 3 so the term is constant within a
//                         group of eight rows).
// A bijection: the XOR term depends on i >> 3 only.
struct Swz {
  int hs;
  __device__ __forceinline__ explicit Swz(const FshtRingFFT& rf)
      : hs(rf.logT > 9 ? rf.logT - 6 : 3) {}
  __device__ __forceinline__ int operator()(int i) const {
    const int r = i >> 3;
    return i ^ ((r ^ ((r & 2) << 1) ^ (r >> hs)) & 7);
  }
};

// In-place decimation-in-frequency FFT of rf.P points in shared memory, natural order in,
// transform order out: an optional radix-3 pass (P = 3 T) splits the data into three
// blocks of T = 2^logT, then radix-4 passes (radix-2^2 butterflies: three twiddles, none
// in the last pass) and a radix-2 pass when logT is odd.  A power-of-two transform
// leaves bin q at bit-reverse(q).  Inputs at nz and above are zero (Bluestein's padding):
// the first pass then skips the products with them (exact, the same results).  All threads of
// the block call it; it synchronises on entry and after every pass.
template <class E>
__device__ void fft_dif(E* buf, const FshtRingFFT& rf, const FftTwT<E>& tw, int nz,
                        bool last = true) {
  using namespace fftp;
  const Swz S(rf);
  constexpr bool kF64 = std::is_same<E, double2>::value;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int logT = rf.logT, T = 1 << logT;
  const int nblk = rf.r3 ? 3 : 1;
  __syncthreads();   // the caller's writes to buf must land first
  if (rf.r3) {
    const E* t3 = tw.r3 + 2 * (T - 1);
    const bool c_zero = nz <= 2 * T;   // the third input of every butterfly is padding
    for (int j = tid; j < T; j += nt) {
      const E a = buf[S(j)], b = buf[S(j + T)];
      const E c = c_zero ? zero_e<E>() : buf[S(j + 2 * T)];
      const E sm = c_zero ? b : ladd(b, c), df = c_zero ? b : lsub(b, c);
      E y1, y2;
      // w3 = exp(-2 pi i / 3): a + w3 b + w3^2 c = t - i (sqrt3/2) df, the other t + i ...
      if constexpr (kF64) {
        const double2 t = make_double2(fma(-0.5, sm.x, a.x), fma(-0.5, sm.y, a.y));
        y1 = make_double2(fma(kSqrt3Half, df.y, t.x), fma(-kSqrt3Half, df.x, t.y));
        y2 = make_double2(fma(-kSqrt3Half, df.y, t.x), fma(kSqrt3Half, df.x, t.y));
      } else {
        const cdd t = lsub(a, cscale_p2(sm, 0.5f));
        const cdd u = cmul_pi(cscale_dd(df, kSqrt3HalfHi, kSqrt3HalfLo));
        y1 = lsub(t, u);
        y2 = ladd(t, u);
      }
      buf[S(j)] = fin(ladd(a, sm));
      buf[S(j + T)] = fin(lmul(y1, ldg_e(&t3[2 * j])));
      buf[S(j + 2 * T)] = fin(lmul(y2, ldg_e(&t3[2 * j + 1])));
    }
    __syncthreads();
  }
  int logspan = logT;
  // last = false: stop before the twiddle-free last pass (span 4 or 2), which the caller
  // fuses with what follows
  const int stop = (last || (logT & 1)) ? 2 : 4;
  for (; logspan >= stop; logspan -= 2) {
    const int lh = logspan - 2, h = 1 << lh;
    const int per_blk = 1 << (logT - 2);
    const E* t4 = tw.r4 + 3 * ((1 << logspan) - 8) / 4;   // used when h > 1
    // first pass over zero-padded data: the inputs at i0 + 2h, i0 + 3h are all padding
    const bool cd_zero = !rf.r3 && logspan == logT && nz <= 2 * h;
    for (int idx = tid; idx < nblk * per_blk; idx += nt) {
      const int blk = idx >> (logT - 2);
      const int r = idx & (per_blk - 1);
      const int j = r & (h - 1);
      const int i0 = (blk << logT) + ((r >> lh) << logspan) + j;
      E apc, amc, bpd, bmd;
      if (cd_zero) {
        apc = amc = buf[S(i0)];
        bpd = bmd = buf[S(i0 + h)];
      } else {
        const E a = buf[S(i0)], b = buf[S(i0 + h)], c = buf[S(i0 + 2 * h)],
                d = buf[S(i0 + 3 * h)];
        apc = ladd(a, c);
        amc = lsub(a, c);
        bpd = ladd(b, d);
        bmd = lsub(b, d);
      }
      const E y1 = lsub(apc, bpd);
      const E mib = cmul_mi(bmd);
      const E y2 = ladd(amc, mib);   // (a-c) - i(b-d)
      const E y3 = lsub(amc, mib);   // (a-c) + i(b-d)
      buf[S(i0)] = fin(ladd(apc, bpd));
      if (h == 1) {
        buf[S(i0 + h)] = fin(y1);
        buf[S(i0 + 2 * h)] = fin(y2);
        buf[S(i0 + 3 * h)] = fin(y3);
      } else {
        buf[S(i0 + h)] = fin(lmul(y1, ldg_e(&t4[3 * j + 1])));
        buf[S(i0 + 2 * h)] = fin(lmul(y2, ldg_e(&t4[3 * j])));
        buf[S(i0 + 3 * h)] = fin(lmul(y3, ldg_e(&t4[3 * j + 2])));
      }
    }
    __syncthreads();
  }
  if (logspan == 1 && last) {
    for (int idx = tid; idx < nblk << (logT - 1); idx += nt) {
      const E a = buf[S(2 * idx)], b = buf[S(2 * idx + 1)];
      buf[S(2 * idx)] = fin(ladd(a, b));
      buf[S(2 * idx + 1)] = fin(lsub(a, b));
    }
    __syncthreads();
  }
}

// The inverse of fft_dif without normalisation (P times the inverse DFT): transform order
// in, natural order out; the passes of fft_dif in reverse with conjugate twiddles.  Only the
// outputs below nout are wanted (Bluestein keeps nd of P): the last pass skips the others.
template <class E>
__device__ void fft_dit_inv(E* buf, const FshtRingFFT& rf, const FftTwT<E>& tw, int nout,
                            bool first = true) {
  using namespace fftp;
  const Swz S(rf);
  constexpr bool kF64 = std::is_same<E, double2>::value;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int logT = rf.logT, T = 1 << logT;
  const int nblk = rf.r3 ? 3 : 1;
  __syncthreads();
  // first = false: the twiddle-free first pass (span 2 or 4) was fused into the caller's
  // previous step
  int logspan = 2;
  if (logT & 1) {
    if (first) {
      for (int idx = tid; idx < nblk << (logT - 1); idx += nt) {
        const E a = buf[S(2 * idx)], b = buf[S(2 * idx + 1)];
        buf[S(2 * idx)] = fin(ladd(a, b));
        buf[S(2 * idx + 1)] = fin(lsub(a, b));
      }
      __syncthreads();
    }
    logspan = 3;
  } else if (!first) {
    logspan = 4;
  }
  for (; logspan <= logT; logspan += 2) {
    const int lh = logspan - 2, h = 1 << lh;
    const int per_blk = 1 << (logT - 2);
    const E* t4 = tw.r4 + 3 * ((1 << logspan) - 8) / 4;   // used when h > 1
    const bool low_half = !rf.r3 && logspan == logT && nout <= 2 * h;   // outputs < 2h only
    for (int idx = tid; idx < nblk * per_blk; idx += nt) {
      const int blk = idx >> (logT - 2);
      const int r = idx & (per_blk - 1);
      const int j = r & (h - 1);
      const int i0 = (blk << logT) + ((r >> lh) << logspan) + j;
      const E y0 = buf[S(i0)];
      const E y1 = buf[S(i0 + h)], y2 = buf[S(i0 + 2 * h)], y3 = buf[S(i0 + 3 * h)];
      E sp, dm, e, f;
      if (h > 1) {
        const E w1 = ldg_e(&t4[3 * j]);
        const E w2 = ldg_e(&t4[3 * j + 1]);
        const E w3 = ldg_e(&t4[3 * j + 2]);
        if constexpr (kF64) {
          // twiddles folded into the adds: sp = y0 + conj(w2) y1 and e = conj(w1) y2 +
          // conj(w3) y3 as FMA chains, dm = 2 y0 - sp, f = 2 z2 - e (24 FP64 ops, not 28)
          sp = make_double2(fma(w2.x, y1.x, fma(w2.y, y1.y, y0.x)),
                            fma(w2.x, y1.y, fma(-w2.y, y1.x, y0.y)));
          dm = make_double2(fma(2.0, y0.x, -sp.x), fma(2.0, y0.y, -sp.y));
          const double2 z2 = cmul(y2, cconj(w1));
          e = make_double2(fma(w3.x, y3.x, fma(w3.y, y3.y, z2.x)),
                           fma(w3.x, y3.y, fma(-w3.y, y3.x, z2.y)));
          f = make_double2(fma(2.0, z2.x, -e.x), fma(2.0, z2.y, -e.y));
        } else {
          const E z1 = lmulc(y1, w2), z2 = lmulc(y2, w1), z3 = lmulc(y3, w3);
          sp = ladd(y0, z1);
          dm = lsub(y0, z1);
          e = ladd(z2, z3);
          f = lsub(z2, z3);
        }
      } else {
        sp = ladd(y0, y1);
        dm = lsub(y0, y1);
        e = ladd(y2, y3);
        f = lsub(y2, y3);
      }
      const E mif = cmul_mi(f);
      buf[S(i0)] = fin(ladd(sp, e));
      buf[S(i0 + h)] = fin(lsub(dm, mif));         // d + i f
      if (!low_half) {
        buf[S(i0 + 2 * h)] = fin(lsub(sp, e));
        buf[S(i0 + 3 * h)] = fin(ladd(dm, mif));   // d - i f
      }
    }
    __syncthreads();
  }
  if (rf.r3) {
    const E* t3 = tw.r3 + 2 * (T - 1);
    const bool two_blocks = nout <= 2 * T;   // the third block is not wanted
    for (int j = tid; j < T; j += nt) {
      const E a = buf[S(j)];
      const E b = lmulc(buf[S(j + T)], ldg_e(&t3[2 * j]));
      const E c = lmulc(buf[S(j + 2 * T)], ldg_e(&t3[2 * j + 1]));
      const E sm = ladd(b, c), df = lsub(b, c);
      buf[S(j)] = fin(ladd(a, sm));
      if constexpr (kF64) {
        const double2 t = make_double2(fma(-0.5, sm.x, a.x), fma(-0.5, sm.y, a.y));
        buf[S(j + T)] = make_double2(fma(-kSqrt3Half, df.y, t.x), fma(kSqrt3Half, df.x, t.y));
        if (!two_blocks)
          buf[S(j + 2 * T)] = make_double2(fma(kSqrt3Half, df.y, t.x), fma(-kSqrt3Half, df.x, t.y));
      } else {
        const cdd t = lsub(a, cscale_p2(sm, 0.5f));
        const cdd u = cmul_pi(cscale_dd(df, kSqrt3HalfHi, kSqrt3HalfLo));
        buf[S(j + T)] = fin(ladd(t, u));
        if (!two_blocks) buf[S(j + 2 * T)] = fin(lsub(t, u));
      }
    }
    __syncthreads();
  }
}

// Where bin q of ring_dft's output sits in buf.
__device__ __forceinline__ int dft_bin(const FshtRingFFT& rf, int q) {
  return rf.bluestein ? q : (int)(__brev((unsigned)q) >> (32 - rf.logT));
}

// DFT of rf.nd points (in buf[0..nd)), forward (e^{-2 pi i jk/nd}); bin q lands at
// buf[dft_bin(rf, q)].  A power-of-two ring is one fft_dif; any other length uses
// Bluestein with the ring's chirp and filter spectrum (transform order, divided by P):
// chirp, fft_dif, filter, fft_dit_inv, chirp, natural order out.
template <class E>
__device__ void ring_dft(E* buf, const FshtRingFFT& rf, const FftTwT<E>& tw,
                         const E* __restrict__ chirp, const E* __restrict__ bhat) {
  using namespace fftp;
  const Swz S(rf);
  const int tid = threadIdx.x, nt = blockDim.x;
  if (!rf.bluestein) {
    fft_dif(buf, rf, tw, rf.P);
    return;
  }
  const int n = rf.nd, P = rf.P;
  for (int j = tid; j < P; j += nt) {
    if (j < n) buf[S(j)] = fin(lmul(buf[S(j)], ldg_e(&chirp[j])));
    else buf[S(j)] = zero_e<E>();
  }
  fft_dif(buf, rf, tw, n, false);
  // the forward transform's twiddle-free last pass, the filter and the inverse's
  // twiddle-free first pass, on the same 4 (odd log2: 2) elements in registers
  if (!(rf.logT & 1)) {
    for (int idx = tid; idx < (P >> 2); idx += nt) {
      const int i0 = 4 * idx;
      const E a = buf[S(i0)], b = buf[S(i0 + 1)], c = buf[S(i0 + 2)], d = buf[S(i0 + 3)];
      const E apc = ladd(a, c), amc = lsub(a, c), bpd = ladd(b, d), bmd = lsub(b, d);
      const E mib = cmul_mi(bmd);
      const E y0 = fin(lmul(ladd(apc, bpd), ldg_e(&bhat[i0])));
      const E y1 = fin(lmul(lsub(apc, bpd), ldg_e(&bhat[i0 + 1])));
      const E y2 = fin(lmul(ladd(amc, mib), ldg_e(&bhat[i0 + 2])));
      const E y3 = fin(lmul(lsub(amc, mib), ldg_e(&bhat[i0 + 3])));
      const E sp = ladd(y0, y1), dm = lsub(y0, y1), e = ladd(y2, y3), f = lsub(y2, y3);
      const E mif = cmul_mi(f);
      buf[S(i0)] = fin(ladd(sp, e));
      buf[S(i0 + 1)] = fin(lsub(dm, mif));
      buf[S(i0 + 2)] = fin(lsub(sp, e));
      buf[S(i0 + 3)] = fin(ladd(dm, mif));
    }
  } else {
    for (int idx = tid; idx < (P >> 1); idx += nt) {
      const int i0 = 2 * idx;
      const E a = buf[S(i0)], b = buf[S(i0 + 1)];
      const E y0 = fin(lmul(ladd(a, b), ldg_e(&bhat[i0])));
      const E y1 = fin(lmul(lsub(a, b), ldg_e(&bhat[i0 + 1])));
      buf[S(i0)] = fin(ladd(y0, y1));
      buf[S(i0 + 1)] = fin(lsub(y0, y1));
    }
  }
  fft_dit_inv(buf, rf, tw, n, false);
  for (int j = tid; j < n; j += nt) buf[S(j)] = fin(lmul(buf[S(j)], ldg_e(&chirp[j])));
  __syncthreads();
}

// ------------------------------------------------------------------ synthesis spectra (FP64)
// Bin q of the packed spectrum Z[q] = Y_N[q] + i Y_S[q] of a ring pair from G_m (north, W[0])
// and G_m(i') (south, W[1]), m <= mtop, with ph[m] = e^{i m phi0}:
//   Y[q] = sum_{m = q mod n} (c_m/2) G_m e^{i m phi0} + sum_{m = -q mod n} (c_m/2) conj(G_m e^{i m phi0}),
// c_0 = 1, c_{m>0} = 2 (the reference's mat2fft_fast, src/fft_mapping.f90:84-128).
__device__ __forceinline__ double2 packed_spectrum_bin(const double2* ph,
                                                       const double2* __restrict__ W,
                                                       long long stride_m, int n, int mtop,
                                                       bool equator, int q) {
  double2 yN = make_double2(0.0, 0.0), yS = make_double2(0.0, 0.0);
  // m = q (mod n)
  for (int m = q; m <= mtop; m += n) {
    const double2* w = W + (long long)m * stride_m;
    const double c = (m == 0) ? 0.5 : 1.0;
    yN = cadd(yN, cscale(cmul(ph[m], w[0]), c));
    if (!equator) yS = cadd(yS, cscale(cmul(ph[m], w[1]), c));
  }
  // m = -q (mod n)
  const int q2 = (q == 0) ? 0 : n - q;
  for (int m = q2; m <= mtop; m += n) {
    const double2* w = W + (long long)m * stride_m;
    const double c = (m == 0) ? 0.5 : 1.0;
    yN = cadd(yN, cscale(cconj(cmul(ph[m], w[0])), c));
    if (!equator) yS = cadd(yS, cscale(cconj(cmul(ph[m], w[1])), c));
  }
  return make_double2(yN.x - yS.y, yN.y + yS.x);   // Y_N + i Y_S
}

// Bin q of one ring's Hermitian spectrum (side 0: north from G_N, side 1: south from G_S),
// the aliased sum packed_spectrum_bin forms for both rings at once.
__device__ __forceinline__ double2 spectrum_bin(const double2* ph, const double2* __restrict__ W,
                                                long long stride_m, int n, int mtop, int side,
                                                int q) {
  double2 y = make_double2(0.0, 0.0);
  for (int m = q; m <= mtop; m += n) {
    const double c = (m == 0) ? 0.5 : 1.0;
    y = cadd(y, cscale(cmul(ph[m], W[(long long)m * stride_m + side]), c));
  }
  const int q2 = (q == 0) ? 0 : n - q;
  for (int m = q2; m <= mtop; m += n) {
    const double c = (m == 0) ? 0.5 : 1.0;
    y = cadd(y, cscale(cconj(cmul(ph[m], W[(long long)m * stride_m + side])), c));
  }
  return y;
}
