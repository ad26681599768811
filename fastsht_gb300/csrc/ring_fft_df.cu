// Ring FFTs of the split-precision form in df64 arithmetic (df64.cuh).
//
// Same transform, layout and output as the FP64 kernels of ring_fft.cu (the reference's
// map2fft + fft2mat_fast, src/compute_fft.f90:15-280 and src/fft_mapping.f90:19-140): per ring
// pair the packed N + iS DFT, then per m the aliased bin times e^{-i m phi0}, written as
// {S, D} = {F_N + F_S, F_N - F_S} in FP64.  Only the arithmetic differs: each (ring pair, map)
// is scaled by a power of two so that its largest value lies in [1, 2), converted to df64 by
// bit manipulation, transformed on the FP32 pipe (GB300: 64 times the FP64 instruction rate)
// with df64 twiddles, chirps and filter spectra, and converted back with one FP64 addition per
// output value.  The transform's error is about 2^-44 of the ring's largest value, far below
// the split contraction's digit resolution (2^-31 of the column maximum).
#include "common.cuh"
#include "fft_passes.cuh"
#include "fft_r16.cuh"

#include <cmath>

namespace {

struct FwdDfArgs {
  const double* maps;       // chunk base: map k at maps + k * map_stride
  long long map_stride;
  int kc, maps_per_block;   // kc: maps in the chunk (the map stride of W)
  int k_off, k_cnt;         // the maps of this launch: [k_off, k_off + k_cnt)
  int nside, lmax, nnorth, nring, ring_base;
  const FshtRingFFT* rfs;
  FftTwT<cdd> tw;            // tw.r3: the radix-3 twiddles
  const cdd* tw16;           // the radix-16 passes' twiddles (fft_r16.cuh)
  const cdd* chirp;
  const cdd* bhat;
  const cdd* rtw;
  const int* ring_i0;
  double2* W;
};

__device__ __forceinline__ cdd cdd_from_fp64(double re, double im) {
  cdd r;
  r.h.x = __double2float_rn(re);
  r.h.y = __double2float_rn(im);
  r.l.x = __double2float_rn(re - (double)r.h.x);
  r.l.y = __double2float_rn(im - (double)r.h.y);
  return r;
}

__device__ __forceinline__ cdd cdd_from_raw(double2 v, int sh) {
  const float2 re = dd_from_double(v.x, sh), im = dd_from_double(v.y, sh);
  cdd r;
  r.h = make_float2(re.x, im.x);
  r.l = make_float2(re.y, im.y);
  return r;
}

__device__ __forceinline__ double2 cdd_to_fp64(cdd v, int sh) {
  if (sh >= -896 && sh <= 896) {   // uniform per (ring pair, map): the short conversion
    const unsigned e896 = (unsigned)(896 + sh) << 20;
    return make_double2(dd_to_double_near(v.h.x, v.l.x, sh, e896),
                        dd_to_double_near(v.h.y, v.l.y, sh, e896));
  }
  return make_double2(dd_to_double(v.h.x, v.l.x, sh), dd_to_double(v.h.y, v.l.y, sh));
}

__device__ __forceinline__ double dd_out(float h, float l, int sh) {
  if (sh >= -896 && sh <= 896) return dd_to_double_near(h, l, sh, (unsigned)(896 + sh) << 20);
  return dd_to_double(h, l, sh);
}

// Loads one ring pair (or one half-length ring) of map values into the FFT buffer's slots as
// raw FP64 pairs, takes the block-wide largest exponent field, then converts every slot to
// df64 scaled by 2^-sh (sh = that exponent, unbiased; 0 for an all-zero ring).  The barrier
// that publishes the exponent also orders the raw stores before the conversion pass, in which
// thread t converts slots t, t + nt, ... in place.  emax is a shared slot that is zero on
// entry.  Returns sh.
template <class Sw>
__device__ __forceinline__ int load_scaled(cdd* buf, const Sw& S, int cnt, const double* xa,
                                           const double* xb, int stride, int* emax) {
  double2* raw = reinterpret_cast<double2*>(buf);
  const int tid = threadIdx.x, nt = blockDim.x;
  int em = 0;
  // Loads unrolled so that several are in flight per thread (the maps may be host memory read
  // over the host link, with microseconds of latency), 16 bytes each where the ring lies on
  // 16-byte boundaries (ring starts are even pixel indices; a caller's map view may not be).
  const bool a16 = ((reinterpret_cast<unsigned long long>(xa) |
                     reinterpret_cast<unsigned long long>(xb)) & 15) == 0;
  if (stride == 2 && xb == xa + 1 && a16) {
    // half-length ring: (x[2j], x[2j + 1]) is one 16-byte load
    const double2* x2 = reinterpret_cast<const double2*>(xa);
#pragma unroll 4
    for (int j = tid; j < cnt; j += nt) {
      const double2 v = __ldg(&x2[j]);
      em = max(em, max(dd_exp_field(v.x), dd_exp_field(v.y)));
      raw[S(j)] = v;
    }
  } else if (stride == 1 && (cnt & 1) == 0 && a16) {
    // ring pair: two consecutive samples of each ring per load
    const double2* a2 = reinterpret_cast<const double2*>(xa);
    const double2* b2 = reinterpret_cast<const double2*>(xb);
#pragma unroll 4
    for (int j = tid; j < cnt / 2; j += nt) {
      const double2 va = __ldg(&a2[j]);
      const double2 vb = xb ? __ldg(&b2[j]) : make_double2(0.0, 0.0);
      em = max(em, max(max(dd_exp_field(va.x), dd_exp_field(va.y)),
                       max(dd_exp_field(vb.x), dd_exp_field(vb.y))));
      raw[S(2 * j)] = make_double2(va.x, vb.x);
      raw[S(2 * j + 1)] = make_double2(va.y, vb.y);
    }
  } else {
#pragma unroll 4
    for (int j = tid; j < cnt; j += nt) {
      const double va = __ldg(&xa[(long long)stride * j]);
      const double vb = xb ? __ldg(&xb[(long long)stride * j]) : 0.0;
      em = max(em, max(dd_exp_field(va), dd_exp_field(vb)));
      raw[S(j)] = make_double2(va, vb);
    }
  }
  em = __reduce_max_sync(0xffffffffu, em);
  if ((tid & 31) == 0) atomicMax(emax, em);
  __syncthreads();
  const int e = *emax;
  const int sh = (e == 0 || e == 0x7ff) ? 0 : e - 1023;
  for (int j = tid; j < cnt; j += nt) buf[S(j)] = cdd_from_raw(raw[S(j)], sh);
  return sh;
}

// The pass flavour of a df64 ring-FFT kernel.  Radix-16 register passes (fft_r16.cuh) execute
// about a fifth fewer instructions but need 128 registers a thread and give a transform P/16
// butterflies per pass: they pay where transforms are large (the belt's 4096 points and the
// large Bluestein sizes).  Segments of small transforms keep the radix-4 passes
// (fft_passes.cuh), whose four times more butterflies per pass keep 512 threads busy at 64
// registers.
template <bool R16>
struct DfPasses {
  using Sw = Swz16;
  template <bool GEN = true>
  static __device__ __forceinline__ void dft(cdd* buf, const FshtRingFFT& rf, const Sw& S,
                                             const FftTwT<cdd>& tw, const cdd* tw16,
                                             const cdd* chirp, const cdd* bhat) {
    ring_dft16<Sw, GEN>(buf, rf, S, tw16, tw.r3, chirp, bhat);
  }
};
template <>
struct DfPasses<false> {
  using Sw = Swz;
  template <bool GEN = true>
  static __device__ __forceinline__ void dft(cdd* buf, const FshtRingFFT& rf, const Sw&,
                                             const FftTwT<cdd>& tw, const cdd*,
                                             const cdd* chirp, const cdd* bhat) {
    ring_dft(buf, rf, tw, chirp, bhat);
  }
};

// NT threads per CTA, at least MINB CTAs per SM (which sets the register budget: 128 a
// thread for <256, 2> and <512, 1>, 64 for <512, 2> and <1024, 1>).  GEN = false: a segment
// of power-of-two rings only (the belt), built without the Bluestein, radix-3 and half-length
// paths.
template <int NT, int MINB, bool R16, bool GEN = true>
__global__ void __launch_bounds__(NT, MINB) k_ring_fft_fwd_df(FwdDfArgs a) {
  using DP = DfPasses<R16>;
  extern __shared__ float4 smem4[];
  __shared__ int s_emax[2];
  const int i = a.ring_base + blockIdx.x;      // north ring index
  const FshtRingFFT rf = a.rfs[i];
  const typename DP::Sw S(rf);
  const int n = rf.n;
  cdd* buf = reinterpret_cast<cdd*>(smem4);    // rf.P entries
  cdd* ph = buf + rf.P;                        // lmax+1 phase factors exp(-i m phi0) / 2
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool equator = (i == a.nnorth - 1);
  const int ip = a.nring - 1 - i;
  const long long off_n = ring_start(a.nside, i);
  const long long off_s = ring_start(a.nside, ip);
  const int sflag = ring_phase_flag(a.nside, i);
  int mtop = a.lmax;
  while (mtop >= 0 && a.ring_i0[mtop] > i) --mtop;
  for (int m = tid; m <= mtop; m += nt) {
    double s = 0.0, c = 1.0;
    if (sflag) {
      long long r = (long long)m % (2LL * n);
      sincospi(-(double)r / (double)n, &s, &c);
    }
    ph[m] = cdd_from_fp64(0.5 * c, 0.5 * s);   // the 1/2 of the N/S split folded in
  }
  if (tid < 2) s_emax[tid] = 0;
  const int k_begin = a.k_off + blockIdx.y * a.maps_per_block;
  const int k_end = min(a.k_off + a.k_cnt, k_begin + a.maps_per_block);
  const cdd* chirp = a.chirp + rf.chirp_off;
  const cdd* bhat = a.bhat + rf.bhat_off;
  int it = 0;   // exponent slot parity: slot it & 1 collects, the other is reset
  if (GEN && rf.nd != n) {
    // Half-length ring (never the equator): each ring as z_j = x_{2j} + i x_{2j+1},
    // Z = DFT_nd(z), X_q = E_q + e^{-2 pi i q/n} O_q (see the FP64 kernel); the north ring
    // writes {F_N, F_N}, the south ring adds +-F_S in FP64.
    const int nd = rf.nd;
    const cdd* rtw = a.rtw + rf.rtw_off;
    for (int k = k_begin; k < k_end; ++k) {
      for (int side = 0; side < 2; ++side, ++it) {
        const double* x = a.maps + (long long)k * a.map_stride + (side ? off_s : off_n);
        __syncthreads();
        if (tid == 0) s_emax[(it & 1) ^ 1] = 0;
        const int sh = load_scaled(buf, S, nd, x, x + 1, 2, &s_emax[it & 1]);
        DP::template dft<GEN>(buf, rf, S, a.tw, a.tw16, chirp, bhat);
        for (int m = tid; m <= mtop; m += nt) {
          const int q = m % n;
          const bool cj = q > nd;
          const int kk = cj ? n - q : q;
          const cdd za = buf[S(dft_bin(rf, kk == nd ? 0 : kk))];
          const cdd zb = cconj(buf[S(dft_bin(rf, kk == 0 ? 0 : nd - kk))]);
          const cdd e = cadd_lz(za, zb);                       // 2 E
          const cdd o = cmul_mi(csub_lz(za, zb));              // 2 O
          cdd xq = cadd_lz(e, cmul_lz(o, ldg_cdd(&rtw[kk])));  // 2 X
          if (cj) xq = cconj(xq);
          const double2 f = cdd_to_fp64(cmul_lz(xq, ph[m]), sh);
          double2* w = a.W + (((long long)m * a.nnorth + i) * a.kc + k) * 2;
          if (side == 0) {
            w[0] = f;
            w[1] = f;
          } else {
            w[0] = cadd(w[0], f);
            w[1] = csub(w[1], f);
          }
        }
      }
    }
    return;
  }
  for (int k = k_begin; k < k_end; ++k, ++it) {
    const double* xn = a.maps + (long long)k * a.map_stride + off_n;
    const double* xs = a.maps + (long long)k * a.map_stride + off_s;
    __syncthreads();   // the previous map's readers of buf and of the other slot are done
    if (tid == 0) s_emax[(it & 1) ^ 1] = 0;
    const int sh = load_scaled(buf, S, n, xn, equator ? nullptr : xs, 1, &s_emax[it & 1]);
    DP::template dft<GEN>(buf, rf, S, a.tw, a.tw16, chirp, bhat);
    // Z = FFT(x_N + i x_S): X_N[q] = (Z[q] + conj Z[-q])/2, X_S[q] = (Z[q] - conj Z[-q])/(2i)
    // q = m mod n and the output pointer advance by fixed steps (no division per m)
    const int qstep = nt % n;
    const long long wstep = (long long)nt * a.nnorth * a.kc * 2;
    int q = tid % n;
    double2* w = a.W + (((long long)tid * a.nnorth + i) * a.kc + k) * 2;
    for (int m = tid; m <= mtop; m += nt, w += wstep) {
      const int qn = (q == 0) ? 0 : n - q;
      const cdd zq = buf[S(dft_bin(rf, q))];
      const cdd zn = cconj(buf[S(dft_bin(rf, qn))]);
      q += qstep;
      if (q >= n) q -= n;
      const cdd xN = cadd_lz(zq, zn);                          // 2 X_N
      const cdd xS = cmul_mi(csub_lz(zq, zn));                 // 2 X_S
      double2 Sv, Dv;   // the {S, D} entries of (m, ring, map)
      if (!sflag) {
        // phi0 = 0: the phase factor is the real 1/2, folded into the output exponent
        if (equator) {
          Sv = Dv = cdd_to_fp64(xN, sh - 1);
        } else {
          Sv = cdd_to_fp64(cadd_lz(xN, xS), sh - 1);
          Dv = cdd_to_fp64(csub_lz(xN, xS), sh - 1);
        }
      } else {
        const cdd p = ph[m];
        if (equator) {
          Sv = Dv = cdd_to_fp64(cmul_lz(xN, p), sh);
        } else {
          Sv = cdd_to_fp64(cmul_lz(cadd_lz(xN, xS), p), sh);  // F_N + F_S
          Dv = cdd_to_fp64(cmul_lz(csub_lz(xN, xS), p), sh);  // F_N - F_S
        }
      }
      w[0] = Sv;
      w[1] = Dv;
    }
  }
}

// ------------------------------------------------------------------ inverse
struct InvDfArgs {
  const double2* W;
  double* maps;
  long long map_stride;
  int kc, maps_per_block;
  int nside, lmax, nnorth, nring, ring_base;
  const FshtRingFFT* rfs;
  FftTwT<cdd> tw;           // tw.r3: the radix-3 twiddles
  const cdd* tw16;          // the radix-16 passes' twiddles (fft_r16.cuh)
  const cdd* chirp;
  const cdd* bhat;
  const double2* rtw;       // FP64: the half-ring combination runs before the conversion
  const int* ring_i0;
};

// The FP64 values the calling thread left in buf's slots [0, cnt) (its own slots t, t + nt,
// ...) become df64 scaled by 2^-sh, sh from the block-wide largest exponent field (em = the
// thread's own largest); conj: store the conjugate.  emax is a shared slot that is zero on
// entry.  Returns sh.
template <class Sw>
__device__ __forceinline__ int convert_scaled(cdd* buf, const Sw& S, int cnt, int em, int* emax,
                                              bool conj) {
  const double2* raw = reinterpret_cast<const double2*>(buf);
  const int tid = threadIdx.x, nt = blockDim.x;
  em = __reduce_max_sync(0xffffffffu, em);
  if ((tid & 31) == 0) atomicMax(emax, em);
  __syncthreads();
  const int e = *emax;
  const int sh = (e == 0 || e == 0x7ff) ? 0 : e - 1023;
  for (int j = tid; j < cnt; j += nt) {
    const double2 v = raw[S(j)];
    buf[S(j)] = cdd_from_raw(conj ? make_double2(v.x, -v.y) : v, sh);
  }
  return sh;
}

__device__ __forceinline__ int exp2f64(double2 v) {
  return max(dd_exp_field(v.x), dd_exp_field(v.y));
}

// Synthesis side of the split form: the spectrum of each ring pair is formed from G in FP64
// (aliasing, x2, e^{+i m phi0}: O(lmax) per ring), scaled and converted to df64, transformed
// as conj(DFT(conj Z)) in df64, and written to the maps with one FP64 addition per pixel.
template <int NT, int MINB, bool R16>
__global__ void __launch_bounds__(NT, MINB) k_ring_fft_inv_df(InvDfArgs a) {
  using DP = DfPasses<R16>;
  extern __shared__ float4 smem4[];
  __shared__ int s_emax[2];
  const int i = a.ring_base + blockIdx.x;
  const FshtRingFFT rf = a.rfs[i];
  const typename DP::Sw S(rf);
  const int n = rf.n;
  cdd* buf = reinterpret_cast<cdd*>(smem4);
  double2* raw = reinterpret_cast<double2*>(smem4);
  double2* ph = reinterpret_cast<double2*>(smem4 + rf.P);   // e^{+i m phi0}, FP64
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool equator = (i == a.nnorth - 1);
  const int ip = a.nring - 1 - i;
  const long long off_n = ring_start(a.nside, i);
  const long long off_s = ring_start(a.nside, ip);
  const int sflag = ring_phase_flag(a.nside, i);
  int mtop = a.lmax;
  while (mtop >= 0 && a.ring_i0[mtop] > i) --mtop;
  for (int m = tid; m <= mtop; m += nt) {
    double s = 0.0, c = 1.0;
    if (sflag) {
      long long r = (long long)m % (2LL * n);
      sincospi((double)r / (double)n, &s, &c);
    }
    ph[m] = make_double2(c, s);
  }
  if (tid < 2) s_emax[tid] = 0;
  const int k_begin = blockIdx.y * a.maps_per_block;
  const int k_end = min(a.kc, k_begin + a.maps_per_block);
  const cdd* chirp = a.chirp + rf.chirp_off;
  const cdd* bhat = a.bhat + rf.bhat_off;
  const long long stride_m = (long long)a.nnorth * a.kc * 2;
  int it = 0;
  if (rf.nd != n) {
    // Half-length ring: x_{2j} + i x_{2j+1} = sum_k Z_k e^{2 pi i jk/nd} with
    // Z_k = (Y_k + Y_{k+nd}) + i (Y_k - Y_{k+nd}) e^{2 pi i k/n}, one ring at a time.
    const int nd = rf.nd;
    const double2* rtw = a.rtw + rf.rtw_off;
    for (int k = k_begin; k < k_end; ++k) {
      const double2* Wk = a.W + ((long long)i * a.kc + k) * 2;
      for (int side = 0; side < 2; ++side, ++it) {
        __syncthreads();
        if (tid == 0) s_emax[(it & 1) ^ 1] = 0;
        int em = 0;
        for (int kk = tid; kk < nd; kk += nt) {
          const double2 y0 = spectrum_bin(ph, Wk, stride_m, n, mtop, side, kk);
          const double2 y1 = spectrum_bin(ph, Wk, stride_m, n, mtop, side, kk + nd);
          const double2 b = cmul(csub(y0, y1), cconj(__ldg(&rtw[kk])));
          const double2 sa = cadd(y0, y1);
          const double2 v = cconj(make_double2(sa.x - b.y, sa.y + b.x));   // conj(A + i B)
          raw[S(kk)] = v;
          em = max(em, exp2f64(v));
        }
        const int sh = convert_scaled(buf, S, nd, em, &s_emax[it & 1], false);
        DP::dft(buf, rf, S, a.tw, a.tw16, chirp, bhat);
        double* x = a.maps + (long long)k * a.map_stride + (side ? off_s : off_n);
        for (int j = tid; j < nd; j += nt) {
          const cdd z = buf[S(dft_bin(rf, j))];   // conj(z): x_{2j} = Re, x_{2j+1} = -Im
          x[2 * j] = dd_out(z.h.x, z.l.x, sh);
          x[2 * j + 1] = -dd_out(z.h.y, z.l.y, sh);
        }
      }
    }
    return;
  }
  for (int k = k_begin; k < k_end; ++k, ++it) {
    const double2* Wk = a.W + ((long long)i * a.kc + k) * 2;
    __syncthreads();
    if (tid == 0) s_emax[(it & 1) ^ 1] = 0;
    int em = 0;
    for (int q = tid; q < n; q += nt) {
      const double2 z = packed_spectrum_bin(ph, Wk, stride_m, n, mtop, equator, q);
      raw[S(q)] = z;
      em = max(em, exp2f64(z));
    }
    // inverse DFT = conj(DFT(conj Z))
    const int sh = convert_scaled(buf, S, n, em, &s_emax[it & 1], true);
    DP::dft(buf, rf, S, a.tw, a.tw16, chirp, bhat);
    double* xn = a.maps + (long long)k * a.map_stride + off_n;
    double* xs = a.maps + (long long)k * a.map_stride + off_s;
    for (int j = tid; j < n; j += nt) {
      const cdd z = buf[S(dft_bin(rf, j))];   // x_N = Re, x_S = -Im of the DFT
      xn[j] = dd_out(z.h.x, z.l.x, sh);
      if (!equator) xs[j] = -dd_out(z.h.y, z.l.y, sh);
    }
  }
}

__global__ void k_to_cdd(const double2* __restrict__ in, float4* out, long long n) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    const double2 v = in[j];
    const cdd c = cdd_from_fp64(v.x, v.y);
    out[j] = make_float4(c.h.x, c.h.y, c.l.x, c.l.y);
  }
}

// Kernel variant of ring segment sgi: radix-16 passes when every transform of the segment has
// at least 4096 points (the belt at nside >= 1024, the large Bluestein caps), with the
// autotuned thread count (256 or 512) or else 512 for one CTA per SM and 256 for two (sixteen
// warps an SM either way); radix-4 passes otherwise, 1024 threads for one CTA per SM and 512
// for two (32 warps).
// pow2_ok: the launcher has the power-of-two-only radix-16 kernels (kR16T*P), used for segments
// without Bluestein, radix-3 or half-length rings.
enum DfVariant { kR16T256, kR16T512, kR4T512, kR4T1024, kR16T256P, kR16T512P };
DfVariant df_variant(const fsht_plan* p, int sgi, bool pow2_ok) {
  const long long smem = p->fft_seg[3 * sgi + 2];
  const bool one_cta = smem > 112 * 1024;
  if (p->fft_seg_pmin[sgi] >= 4096) {
    const bool t512 = p->fft_threads > 0 ? p->fft_threads > 256 : one_cta;
    if (pow2_ok && !p->fft_seg_gen[sgi]) return t512 ? kR16T512P : kR16T256P;
    return t512 ? kR16T512 : kR16T256;
  }
  return one_cta ? kR4T1024 : kR4T512;
}

template <class Args>
int df_set_smem(void (*k)(Args), size_t smem) {
  return fsht_smem_limit((const void*)k, smem);
}

template <class Args>
int df_launch(DfVariant v, void (*const* ks)(Args), dim3 grid, size_t smem, cudaStream_t s,
              const Args& a) {
  static const int threads[6] = {256, 512, 512, 1024, 256, 512};
  ks[v]<<<grid, threads[v], smem, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

// The radix-16 twiddle table (fft_r16.cuh layout), FP64 sincospi of the exactly reduced
// argument, stored as df64
__global__ void k_twiddles16(float4* out, int logTmax) {
  const long long n = fsht_tw16_entries(1 << logTmax);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    int s = 5;
    while (s < logTmax && e >= fsht_tw16_off(s + 1)) ++s;
    const long long loc = e - fsht_tw16_off(s);
    const long long h = 1LL << (s - 4);
    const long long k = loc / h + 1, j = loc % h;
    const long long r = (j * k) & ((1LL << s) - 1);   // j k mod 2^s
    double sn, cs;
    sincospi(-2.0 * (double)r / (double)(1LL << s), &sn, &cs);
    const cdd c = cdd_from_fp64(cs, sn);
    out[e] = make_float4(c.h.x, c.h.y, c.l.x, c.l.y);
  }
}

int to_cdd(const double2* in, float4** out, long long n, cudaStream_t s) {
  const long long cnt = n > 0 ? n : 1;
  FSHT_CUDA_TRY(cudaMalloc(out, sizeof(float4) * cnt));
  if (n > 0) {
    long long g = (n + 255) / 256;
    if (g > 4096) g = 4096;
    k_to_cdd<<<(unsigned)g, 256, 0, s>>>(in, *out, n);
    FSHT_LAUNCH_CHECK();
  }
  return FSHT_OK;
}

}  // namespace

int fsht_fft_df_tables_init(fsht_plan* p) {
  FSHT_TRY(to_cdd(p->d_tw, &p->d_tw_df, fsht_tw_entries(p->Tmax, p->P3max), p->stream));
  FSHT_TRY(to_cdd(p->d_chirp, &p->d_chirp_df, p->fft_chirp_total, p->stream));
  FSHT_TRY(to_cdd(p->d_bhat, &p->d_bhat_df, p->fft_bhat_total, p->stream));
  FSHT_TRY(to_cdd(p->d_rtw, &p->d_rtw_df, p->fft_rtw_total, p->stream));
  const long long n16 = fsht_tw16_entries(p->Tmax);
  FSHT_CUDA_TRY(cudaMalloc(&p->d_tw16_df, sizeof(float4) * (n16 > 0 ? n16 : 1)));
  if (n16 > 0) {
    long long g = (n16 + 255) / 256;
    if (g > 4096) g = 4096;
    k_twiddles16<<<(unsigned)g, 256, 0, p->stream>>>(p->d_tw16_df, p->logTmax);
    FSHT_LAUNCH_CHECK();
  }
  FSHT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  return FSHT_OK;
}

int fsht_launch_ring_fft_fwd_df(fsht_plan* p, const double* maps, long long map_stride, int kc,
                                int k0, int kb, double2* W, cudaStream_t s) {
  FwdDfArgs a;
  a.maps = maps;
  a.map_stride = map_stride;
  a.kc = kc;
  a.k_off = k0;
  a.k_cnt = kb;
  a.nside = p->nside;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.nring = p->nring;
  a.ring_base = 0;
  a.rfs = p->d_rfft;
  a.tw.r4 = reinterpret_cast<const cdd*>(p->d_tw_df);
  a.tw.r3 = reinterpret_cast<const cdd*>(p->d_tw_df) + fsht_tw_r4_entries(p->Tmax);
  a.chirp = reinterpret_cast<const cdd*>(p->d_chirp_df);
  a.bhat = reinterpret_cast<const cdd*>(p->d_bhat_df);
  a.rtw = reinterpret_cast<const cdd*>(p->d_rtw_df);
  a.tw16 = reinterpret_cast<const cdd*>(p->d_tw16_df);
  a.ring_i0 = p->d_ring_i0;
  a.W = W;
  a.maps_per_block = p->fft_mpb > 0 ? p->fft_mpb : fsht_fft_maps_per_block(kb, p->nnorth);
  void (*const ks[6])(FwdDfArgs) = {k_ring_fft_fwd_df<256, 2, true>, k_ring_fft_fwd_df<512, 1, true>,
                                    k_ring_fft_fwd_df<512, 2, false>,
                                    k_ring_fft_fwd_df<1024, 1, false>,
                                    k_ring_fft_fwd_df<256, 2, true, false>,
                                    k_ring_fft_fwd_df<512, 1, true, false>};
  for (auto k : ks) FSHT_TRY(df_set_smem(k, p->fft_smem));
  for (int sgi = 0; sgi < p->fft_nseg; ++sgi) {
    const long long* sg = p->fft_seg + 3 * sgi;
    a.ring_base = (int)sg[0];
    dim3 grid((unsigned)(sg[1] - sg[0]), (kb + a.maps_per_block - 1) / a.maps_per_block);
    FSHT_TRY(df_launch(df_variant(p, sgi, true), ks, grid, (size_t)sg[2], s, a));
  }
  return FSHT_OK;
}

int fsht_launch_ring_fft_inv_df(fsht_plan* p, const double2* W, double* maps,
                                long long map_stride, int kc, cudaStream_t s) {
  InvDfArgs a;
  a.W = W;
  a.maps = maps;
  a.map_stride = map_stride;
  a.kc = kc;
  a.nside = p->nside;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.nring = p->nring;
  a.ring_base = 0;
  a.rfs = p->d_rfft;
  a.tw.r4 = reinterpret_cast<const cdd*>(p->d_tw_df);
  a.tw.r3 = reinterpret_cast<const cdd*>(p->d_tw_df) + fsht_tw_r4_entries(p->Tmax);
  a.chirp = reinterpret_cast<const cdd*>(p->d_chirp_df);
  a.bhat = reinterpret_cast<const cdd*>(p->d_bhat_df);
  a.rtw = p->d_rtw;
  a.tw16 = reinterpret_cast<const cdd*>(p->d_tw16_df);
  a.ring_i0 = p->d_ring_i0;
  a.maps_per_block = p->fft_mpb > 0 ? p->fft_mpb : fsht_fft_maps_per_block(kc, p->nnorth);
  void (*const ks[4])(InvDfArgs) = {k_ring_fft_inv_df<256, 2, true>, k_ring_fft_inv_df<512, 1, true>,
                                    k_ring_fft_inv_df<512, 2, false>,
                                    k_ring_fft_inv_df<1024, 1, false>};
  for (auto k : ks) FSHT_TRY(df_set_smem(k, p->fft_smem));
  for (int sgi = 0; sgi < p->fft_nseg; ++sgi) {
    const long long* sg = p->fft_seg + 3 * sgi;
    a.ring_base = (int)sg[0];
    dim3 grid((unsigned)(sg[1] - sg[0]), (kc + a.maps_per_block - 1) / a.maps_per_block);
    FSHT_TRY(df_launch(df_variant(p, sgi, false), ks, grid, (size_t)sg[2], s, a));
  }
  return FSHT_OK;
}
