// Batched FP64 ring FFTs for HEALPix maps, with the phi0 phase shift, the
// m-aliasing and the north/south folding done in the same pass.
//
// Replaces the reference's map2fft / fft2map (src/compute_fft.f90:15-280, MKL DFTI
// on the host + per-ring PCIe copies) and the per-m gathers fft2mat_fast /
// mat2fft_fast / mat2fft_fast_iter (src/fft_mapping.f90:19-190).
//
// Phase-matrix layout written/read by these kernels ("W"), one per field:
//   W[((m * nnorth + i) * kc + k) * 2 + {0,1}]  (double2)
// for order m <= lmax, north ring i < 2*nside, map k < kc.
//   analysis:  {S, D} = {F_m(i) + F_m(i'), F_m(i) - F_m(i')},  i' = nring-1-i,
//              F_m(i) = sum_j x_{i,j} exp(-i m (phi0_i + 2 pi j / n_i))
//   synthesis: {G_m(i), G_m(i')} with map_{i,j} = Re sum_m c_m G_m(i) e^{i m (phi0 + 2 pi j/n)},
//              c_0 = 1, c_{m>0} = 2.
// The equator ring (i = 2 nside - 1) is its own mirror: S = D = F_m, and only
// G_m(i) is used.
#include "common.cuh"
#include "fft_passes.cuh"
#include <cmath>
#include <vector>
#include <climits>

namespace {

// ------------------------------------------------------------------ tables
// The packed twiddle table (fsht_tw_entries): thread per entry, FP64 sincospi of the exact
// fraction.
__global__ void k_twiddles(double2* tw, int Tmax, int P3max) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n4 = fsht_tw_r4_entries(Tmax);
  if (e >= fsht_tw_entries(Tmax, P3max)) return;
  long long num, den;
  if (e < n4) {
    int s = 3;
    while (3LL * ((2LL << s) - 8) / 4 <= e) ++s;       // span 2^s holds entry e
    const long long r = e - 3LL * ((1LL << s) - 8) / 4;
    num = (r / 3) * (r % 3 + 1);
    den = 1LL << s;
  } else {
    const long long r0 = e - n4;
    int k = 0;
    while (2LL * ((2LL << k) - 1) <= r0) ++k;          // size 3 * 2^k holds entry e
    const long long r = r0 - 2LL * ((1LL << k) - 1);
    num = (r / 2) * (r % 2 + 1);
    den = 3LL << k;
  }
  double sn, cs;
  sincospi(-2.0 * (double)(num % den) / (double)den, &sn, &cs);
  tw[e] = make_double2(cs, sn);
}

// chirp w_j = exp(-i pi j^2 / nd) and the filter spectrum (fft_dif of the wrapped conj
// chirp, over P) for one ring, and a half-length ring's twiddles; block per Bluestein ring.
__global__ void k_bluestein_tables(const FshtRingFFT* rfs, const int* rings, double2* chirp,
                                   double2* bhat, double2* rtw, FftTw tw) {
  extern __shared__ double2 sbuf[];
  const FshtRingFFT rf = rfs[rings[blockIdx.x]];
  const Swz S(rf);
  const int n = rf.nd, P = rf.P;
  if (rf.nd != rf.n) {     // half-length ring: exp(-2 pi i k / n_ring), k <= nd
    for (int k = threadIdx.x; k <= n; k += blockDim.x) {
      double s, c;
      sincospi(-2.0 * (double)k / (double)rf.n, &s, &c);
      rtw[rf.rtw_off + k] = make_double2(c, s);
    }
  }
  double2* w = chirp + rf.chirp_off;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    long long r = ((long long)j * j) % (2LL * n);
    double s, c;
    sincospi(-(double)r / (double)n, &s, &c);
    w[j] = make_double2(c, s);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    double2 v = make_double2(0.0, 0.0);
    if (j < n) v = cconj(w[j]);
    else if (P - j < n) v = cconj(w[P - j]);
    sbuf[S(j)] = v;
  }
  fft_dif(sbuf, rf, tw, rf.P);
  const double invP = 1.0 / (double)P;
  for (int j = threadIdx.x; j < P; j += blockDim.x) bhat[rf.bhat_off + j] = cscale(sbuf[S(j)], invP);
}

// ------------------------------------------------------------------ forward
struct FwdArgs {
  const double* maps;       // chunk base: map k at maps + k * map_stride
  long long map_stride;
  int kc;                   // maps in this chunk (the map stride of W)
  int k_off, k_cnt;         // the maps of this launch: [k_off, k_off + k_cnt)
  int maps_per_block;
  int nside, lmax, nnorth, nring, ring_base;
  const FshtRingFFT* rfs;
  FftTw tw;
  const double2* chirp;
  const double2* bhat;
  const double2* rtw;
  const int* ring_i0;
  double2* W;
};

__global__ void __launch_bounds__(512, 2) k_ring_fft_fwd(FwdArgs a) {
  extern __shared__ double2 smem[];
  const int i = a.ring_base + blockIdx.x;      // north ring index
  const FshtRingFFT rf = a.rfs[i];
  const Swz S(rf);
  const int n = rf.n;
  double2* buf = smem;                          // rf.P entries
  double2* ph = smem + rf.P;                    // lmax+1 phase factors exp(-i m phi0)
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool equator = (i == a.nnorth - 1);
  const int ip = a.nring - 1 - i;
  const long long off_n = ring_start(a.nside, i);
  const long long off_s = ring_start(a.nside, ip);
  const int sflag = ring_phase_flag(a.nside, i);
  // highest m for which ring i is kept (ring_i0 is non-decreasing in m)
  int mtop = a.lmax;
  while (mtop >= 0 && a.ring_i0[mtop] > i) --mtop;   // uniform loop, lmax small-ish
  for (int m = tid; m <= mtop; m += nt) {
    double s = 0.0, c = 1.0;
    if (sflag) {
      long long r = (long long)m % (2LL * n);
      sincospi(-(double)r / (double)n, &s, &c);
    }
    ph[m] = make_double2(0.5 * c, 0.5 * s);    // the 1/2 of the N/S (even/odd) split folded in
  }
  const int k_begin = a.k_off + blockIdx.y * a.maps_per_block;
  const int k_end = min(a.k_off + a.k_cnt, k_begin + a.maps_per_block);
  const double2* chirp = a.chirp + rf.chirp_off;
  const double2* bhat = a.bhat + rf.bhat_off;
  if (rf.nd != n) {
    // Half-length ring (a cap ring whose packed transform exceeds shared memory; never the
    // equator): each of the two rings as z_j = x_{2j} + i x_{2j+1}, Z = DFT_nd(z); then
    // X_q = E_q + e^{-2 pi i q/n} O_q with E = (Z_q + conj Z_{nd-q})/2, O = (Z_q - conj
    // Z_{nd-q})/(2i).  The north ring writes {S, D} = {F_N, F_N}, the south ring adds +-F_S
    // (the same thread owns each m in both passes).
    const int nd = rf.nd;
    const double2* rtw = a.rtw + rf.rtw_off;
    for (int k = k_begin; k < k_end; ++k) {
      for (int side = 0; side < 2; ++side) {
        const double* x = a.maps + (long long)k * a.map_stride + (side ? off_s : off_n);
        __syncthreads();
#pragma unroll 4
        for (int j = tid; j < nd; j += nt)   // unrolled: several loads in flight per thread
          buf[S(j)] = make_double2(__ldg(&x[2 * j]), __ldg(&x[2 * j + 1]));
        __syncthreads();
        ring_dft(buf, rf, a.tw, chirp, bhat);
        for (int m = tid; m <= mtop; m += nt) {
          const int q = m % n;
          const bool cj = q > nd;
          const int kk = cj ? n - q : q;
          const double2 za = buf[S(dft_bin(rf, kk == nd ? 0 : kk))];
          const double2 zb = cconj(buf[S(dft_bin(rf, kk == 0 ? 0 : nd - kk))]);
          const double2 e = cadd(za, zb);                      // 2 E
          const double2 dd = csub(za, zb);
          const double2 o = make_double2(dd.y, -dd.x);         // 2 O
          double2 xq = cadd(e, cmul(__ldg(&rtw[kk]), o));      // 2 X
          if (cj) xq = cconj(xq);
          const double2 f = cmul(ph[m], xq);
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
  for (int k = k_begin; k < k_end; ++k) {
    const double* xn = a.maps + (long long)k * a.map_stride + off_n;
    const double* xs = a.maps + (long long)k * a.map_stride + off_s;
    __syncthreads();
#pragma unroll 4
    for (int j = tid; j < n; j += nt)   // unrolled: several loads in flight per thread
      buf[S(j)] = make_double2(__ldg(&xn[j]), equator ? 0.0 : __ldg(&xs[j]));
    __syncthreads();
    ring_dft(buf, rf, a.tw, chirp, bhat);
    // Z = FFT(x_N + i x_S): X_N[q] = (Z[q] + conj Z[-q])/2, X_S[q] = (Z[q] - conj Z[-q])/(2i)
    for (int m = tid; m <= mtop; m += nt) {
      const int q = m % n;
      const int qn = (q == 0) ? 0 : n - q;
      const double2 zq = buf[S(dft_bin(rf, q))];
      const double2 zn = cconj(buf[S(dft_bin(rf, qn))]);
      const double2 xN = cadd(zq, zn);                         // 2 X_N
      const double2 dd = csub(zq, zn);
      const double2 xS = make_double2(dd.y, -dd.x);            // 2 X_S
      const double2 p = ph[m];                                 // e^{-i m phi0} / 2
      double2* w = a.W + (((long long)m * a.nnorth + i) * a.kc + k) * 2;
      if (equator) {
        const double2 fN = cmul(p, xN);
        w[0] = fN;
        w[1] = fN;
      } else {
        w[0] = cmul(p, cadd(xN, xS));                          // F_N + F_S
        w[1] = cmul(p, csub(xN, xS));                          // F_N - F_S
      }
    }
  }
}

// ------------------------------------------------------------------ inverse
struct InvArgs {
  const double2* W;
  double* maps;
  long long map_stride;
  int kc, maps_per_block;
  int nside, lmax, nnorth, nring, ring_base;
  const FshtRingFFT* rfs;
  FftTw tw;
  const double2* chirp;
  const double2* bhat;
  const double2* rtw;
  const int* ring_i0;
};

// Builds, in buf[0..n), the packed spectrum Z[q] = Y_N[q] + i Y_S[q] of the two
// real rings from G_m (north) and G_m(i') (south), m <= mtop (packed_spectrum_bin).
__device__ void build_spectrum(double2* buf, const Swz& S, const double2* ph,
                               const double2* __restrict__ W, long long stride_m, int n, int mtop,
                               bool equator) {
  for (int q = threadIdx.x; q < n; q += blockDim.x)
    buf[S(q)] = packed_spectrum_bin(ph, W, stride_m, n, mtop, equator, q);
}

__global__ void __launch_bounds__(512, 2) k_ring_fft_inv(InvArgs a) {
  extern __shared__ double2 smem[];
  const int i = a.ring_base + blockIdx.x;
  const FshtRingFFT rf = a.rfs[i];
  const Swz S(rf);
  const int n = rf.n;
  double2* buf = smem;
  double2* ph = smem + rf.P;
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
  const int k_begin = blockIdx.y * a.maps_per_block;
  const int k_end = min(a.kc, k_begin + a.maps_per_block);
  const double2* chirp = a.chirp + rf.chirp_off;
  const double2* bhat = a.bhat + rf.bhat_off;
  const long long stride_m = (long long)a.nnorth * a.kc * 2;
  if (rf.nd != n) {
    // Half-length ring: x_{2j} + i x_{2j+1} = sum_k Z_k e^{2 pi i jk/nd} with
    // Z_k = (Y_k + Y_{k+nd}) + i (Y_k - Y_{k+nd}) e^{2 pi i k/n}, one ring at a time.
    const int nd = rf.nd;
    const double2* rtw = a.rtw + rf.rtw_off;
    for (int k = k_begin; k < k_end; ++k) {
      const double2* Wk = a.W + ((long long)i * a.kc + k) * 2;
      for (int side = 0; side < 2; ++side) {
        __syncthreads();
        for (int kk = tid; kk < nd; kk += nt) {
          const double2 y0 = spectrum_bin(ph, Wk, stride_m, n, mtop, side, kk);
          const double2 y1 = spectrum_bin(ph, Wk, stride_m, n, mtop, side, kk + nd);
          const double2 b = cmul(csub(y0, y1), cconj(__ldg(&rtw[kk])));
          const double2 sa = cadd(y0, y1);
          buf[S(kk)] = cconj(make_double2(sa.x - b.y, sa.y + b.x));   // conj(A + i B)
        }
        __syncthreads();
        ring_dft(buf, rf, a.tw, chirp, bhat);
        double* x = a.maps + (long long)k * a.map_stride + (side ? off_s : off_n);
        for (int j = tid; j < nd; j += nt) {
          const double2 z = buf[S(dft_bin(rf, j))];   // conj(z): x_{2j} = Re, x_{2j+1} = -Im
          x[2 * j] = z.x;
          x[2 * j + 1] = -z.y;
        }
      }
    }
    return;
  }
  for (int k = k_begin; k < k_end; ++k) {
    __syncthreads();
    build_spectrum(buf, S, ph, a.W + ((long long)i * a.kc + k) * 2, stride_m, n, mtop, equator);
    __syncthreads();
    // inverse DFT = conj(DFT(conj Z))
    for (int j = tid; j < n; j += nt) buf[S(j)] = cconj(buf[S(j)]);
    __syncthreads();
    ring_dft(buf, rf, a.tw, chirp, bhat);
    double* xn = a.maps + (long long)k * a.map_stride + off_n;
    double* xs = a.maps + (long long)k * a.map_stride + off_s;
    for (int j = tid; j < n; j += nt) {
      const double2 z = buf[S(dft_bin(rf, j))];   // conj applied: x_N = Re, x_S = -Im of the DFT
      xn[j] = z.x;
      if (!equator) xs[j] = -z.y;
    }
  }
}

// ------------------------------------------------------------------ residual
// Fourier-space residual of the Jacobi iterations (reference mat2fft_fast_iter,
// src/fft_mapping.f90:142-190, read back by fft2mat_fast): for every kept m,
//   F^R_m(i) = F^X_m(i) - n_i e^{-i m phi0} Y_i[m mod n_i],
// where Y_i is the Hermitian spectrum synthesised from G (every m' = +-q mod n_i
// lands in bin q).  X holds {S, D}; GR holds {G_N, G_S} on entry and {S_R, D_R}
// on exit.  prefix = 0 ("old" method, t2alm_iter_old): Y sums all m'.  prefix = 1
// ("new" method, t2alm_iter, sht_main.f90:171-264): the reference forms each
// order's residual right after its own synthesis, so Y only holds m' <= m.
// Thread per half-spectrum bin p in [0, n/2]: it owns every m that lands in p or
// n - p, walks them in ascending order and needs no shared spectrum.
struct ResArgs {
  const double2* X;
  double2* GR;
  int kc, maps_per_block;
  int nside, lmax, nnorth, ring_base, prefix;
  const FshtRingFFT* rfs;
  const int* ring_i0;
};

__global__ void __launch_bounds__(512) k_fourier_residual(ResArgs a) {
  extern __shared__ double2 smem[];
  const int i = a.ring_base + blockIdx.x;
  const int n = a.rfs[i].n;
  double2* phf = smem;   // lmax+1: exp(+i m phi0)
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool equator = (i == a.nnorth - 1);
  const int sflag = ring_phase_flag(a.nside, i);
  int mtop = a.lmax;
  while (mtop >= 0 && a.ring_i0[mtop] > i) --mtop;
  for (int m = tid; m <= mtop; m += nt) {
    double s = 0.0, c = 1.0;
    if (sflag) {
      long long r = (long long)m % (2LL * n);
      sincospi((double)r / (double)n, &s, &c);
    }
    phf[m] = make_double2(c, s);
  }
  __syncthreads();
  const long long stride_m = (long long)a.nnorth * a.kc * 2;
  const int k_begin = blockIdx.y * a.maps_per_block;
  const int k_end = min(a.kc, k_begin + a.maps_per_block);
  const int half = n / 2;
  const double dn = (double)n;
  for (int k = k_begin; k < k_end; ++k) {
    const long long base = ((long long)i * a.kc + k) * 2;
    for (int p = tid; p <= half; p += nt) {
      const int pn = (n - p) % n;     // the mirrored bin (p itself for p = 0, n/2)
      // ascending merge of {p + t n} and {pn + t n}; when p == pn one list
      int ma = p, mb = (pn == p) ? INT_MAX : pn;
      double2 yN = make_double2(0.0, 0.0), yS = make_double2(0.0, 0.0);
      // pass 0 (old method only): totals; pass 1: emit residuals (accumulating
      // the prefix first when prefix = 1)
      for (int pass = a.prefix ? 1 : 0; pass < 2; ++pass) {
        int ua = ma, ub = mb;
        while (true) {
          const int m = min(ua, ub);
          if (m > mtop) break;
          const bool inA = (m == ua);
          if (inA) ua += n; else ub += n;
          const double2* g = a.GR + base + (long long)m * stride_m;
          const double c = (m == 0) ? 0.5 : 1.0;
          const double2 hN = cscale(cmul(phf[m], g[0]), c);
          const double2 hS = equator ? make_double2(0.0, 0.0) : cscale(cmul(phf[m], g[1]), c);
          const int q = m % n;
          // this m adds to bin p: h if q == p, conj(h) if q == n - p (both when p == pn)
          if (pass == 0 || a.prefix) {
            if (q == p) { yN = cadd(yN, hN); yS = cadd(yS, hS); }
            if (q == pn) { yN = cadd(yN, cconj(hN)); yS = cadd(yS, cconj(hS)); }
          }
          if (pass == 1) {
            // Y[q] = Y[p] when q == p, conj(Y[p]) otherwise
            const double2 vN = (q == p) ? yN : cconj(yN);
            const double2 vS = (q == p) ? yS : cconj(yS);
            const double2 e = cconj(phf[m]);
            const double2 rN = cscale(cmul(e, vN), dn);
            const double2* x = a.X + base + (long long)m * stride_m;
            double2* o = a.GR + base + (long long)m * stride_m;
            const double2 x0 = x[0], x1 = x[1];
            if (equator) {
              o[0] = csub(x0, rN);
              o[1] = csub(x1, rN);
            } else {
              const double2 rS = cscale(cmul(e, vS), dn);
              o[0] = csub(x0, cadd(rN, rS));
              o[1] = csub(x1, csub(rN, rS));
            }
          }
        }
      }
    }
  }
}

// ------------------------------------------------------------------ ring skip
// kept(i, m): max_{m <= l <= lcap} |lambda_lm(theta_i)| >= 1e-20, evaluated with the
// exponent-rescaled recursion (values carried as v * 2^(600 e), e <= 0).
__device__ bool ring_kept(double c, double s, double pref, int m, int lcap) {
  int ex;
  double mt = frexp(s, &ex);
  double rm = 1.0, bm = mt;
  long long re = 0, be = ex;
  for (int k = m; k; k >>= 1) {
    if (k & 1) { rm *= bm; re += be; int t; rm = frexp(rm, &t); re += t; }
    if (k > 1) { bm *= bm; be *= 2; int t; bm = frexp(bm, &t); be += t; }
  }
  rm *= pref;
  { int t; rm = frexp(rm, &t); re += t; }
  int e = (re >= -300) ? 0 : (int)floor((double)(re + 300) / 600.0);
  double cur = ldexp(rm, (int)(re - 600LL * e)), prev = 0.0;
  if (e == 0 && fabs(cur) >= 1e-20) return true;
  const double mm = (double)m * (double)m;
  for (int l = m + 1; l <= lcap; ++l) {
    const double dl = (double)l;
    const double al = sqrt((4.0 * dl * dl - 1.0) / (dl * dl - mm));
    const double bl = sqrt(((dl - 1.0) * (dl - 1.0) - mm) / ((2.0 * dl - 3.0) * (2.0 * dl - 1.0))) * al;
    const double nx = al * c * cur - bl * prev;
    prev = cur;
    cur = nx;
    if (e < 0 && fabs(cur) > 0x1p300) { cur *= 0x1p-600; prev *= 0x1p-600; ++e; }
    if (e == 0 && fabs(cur) >= 1e-20) return true;
  }
  return false;
}

// i0(m) = first north ring kept for order m (the rule the reference's
// SHT_ring_skip_table/<nside>.bin follows).  max_l |lambda_lm| grows toward the
// equator, so a binary search over rings suffices; thread per m.  The host makes
// the result non-decreasing in m.
__global__ void k_ring_first_kept(const double* cth, const double* sth, const double* pref,
                                  int nnorth, int lcap, int mmax, int* first) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m > mmax) return;
  int lo = 0, hi = nnorth - 1;     // the equator ring is always kept for m <= lcap
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (ring_kept(cth[mid], sth[mid], pref[m], m, lcap)) hi = mid;
    else lo = mid + 1;
  }
  first[m] = lo;
}

int maps_per_block_for(int kc, int nrings_launched) {
  // aim for >= ~8 blocks per SM over 152 SMs
  long long target = 152LL * 8;
  int g = (int)((long long)kc * nrings_launched / target);
  if (g < 1) g = 1;
  if (g > 16) g = 16;
  return g;
}

}  // namespace

int fsht_fft_maps_per_block(int kc, int nrings) { return maps_per_block_for(kc, nrings); }

// ================================================================== host side
int fsht_fft_layout(int nside, int lmax, FshtFftLayout* lay, FshtRingFFT* rfs, int* blue_rings) {
  const int nn = 2 * nside;
  const size_t smem_cap = 227 * 1024;
  long long chirp_total = 0, bhat_total = 0, rtw_total = 0;
  int Pmax = 4, logTmax = 2, P3max = 0, nblue = 0, nhalf = 0;
  for (int i = 0; i < nn; ++i) {
    FshtRingFFT r{};
    r.n = ring_len(nside, i);
    r.nd = r.n;
    fsht_ring_fft_size(r);
    if (r.bluestein && (size_t)(r.P + lmax + 1) * sizeof(double2) > smem_cap) {
      // the packed N + iS transform does not fit: transform each ring at half length
      r.nd = r.n / 2;
      fsht_ring_fft_size(r);
      r.rtw_off = rtw_total;
      rtw_total += r.nd + 1;
      ++nhalf;
    }
    if (r.bluestein) {
      r.chirp_off = chirp_total;
      r.bhat_off = bhat_total;
      chirp_total += r.nd;
      bhat_total += r.P;
      if (blue_rings) blue_rings[nblue] = i;
      ++nblue;
    }
    if (r.P >= 8 && (r.P & 7)) {
      // the df64 kernels' shared-memory swizzle permutes rows of eight elements; ring lengths
      // 4 (i + 1) and 4 nside never give such a size (the smallest Bluestein size is 24)
      fsht_set_error("ring %d: transform size %d is not a multiple of 8", i, r.P);
      return FSHT_EUNSUPPORTED;
    }
    if (r.P > Pmax) Pmax = r.P;
    if (r.logT > logTmax) logTmax = r.logT;
    if (r.r3 && r.P > P3max) P3max = r.P;
    if (rfs) rfs[i] = r;
  }
  lay->Pmax = Pmax;
  lay->Tmax = 1 << logTmax;
  lay->logTmax = logTmax;
  lay->P3max = P3max;
  lay->chirp_total = chirp_total;
  lay->bhat_total = bhat_total;
  lay->rtw_total = rtw_total;
  lay->nblue = nblue;
  lay->nhalf = nhalf;
  // The phase table (lmax+1) and the FFT buffer (Pmax) share the dynamic smem.
  lay->smem = (size_t)(Pmax + lmax + 1) * sizeof(double2);
  if (lay->smem > smem_cap) {
    fsht_set_error("ring FFT needs %zu bytes of shared memory (nside %d, lmax %d): unsupported",
                   lay->smem, nside, lmax);
    return FSHT_EUNSUPPORTED;
  }
  return FSHT_OK;
}

namespace {
FftTw plan_tw(const fsht_plan* p) {
  FftTw t;
  t.r4 = p->d_tw;
  t.r3 = p->d_tw + fsht_tw_r4_entries(p->Tmax);
  return t;
}
}  // namespace

int fsht_fft_tables_fill(fsht_plan* p, const int* d_blue_rings, int nblue, cudaStream_t s) {
  const long long ntw = fsht_tw_entries(p->Tmax, p->P3max);
  if (ntw > 0) {
    k_twiddles<<<(unsigned)((ntw + 255) / 256), 256, 0, s>>>(p->d_tw, p->Tmax, p->P3max);
  }
  FSHT_LAUNCH_CHECK();
  if (nblue > 0) {
    const size_t sm = (size_t)p->Pmax * sizeof(double2);
    FSHT_TRY(fsht_smem_limit((const void*)k_bluestein_tables, (size_t)(sm)));
    k_bluestein_tables<<<(unsigned)nblue, 512, sm, s>>>(p->d_rfft, d_blue_rings, p->d_chirp,
                                                         p->d_bhat, p->d_rtw, plan_tw(p));
    FSHT_LAUNCH_CHECK();
  }
  return FSHT_OK;
}

int fsht_fft_tables_init(fsht_plan* p) {
  const int nn = p->nnorth;
  std::vector<FshtRingFFT> rfs(nn);
  std::vector<int> blue_rings(nn);
  FshtFftLayout lay;
  int rc = fsht_fft_layout(p->nside, p->lmax, &lay, rfs.data(), blue_rings.data());
  if (rc) return rc;
  {
    // consecutive rings whose (P + lmax + 1) double2 fit twice per SM form one launch segment
    const size_t two_per_sm = 112 * 1024;
    p->fft_nseg = 0;
    int cls_prev = -1;
    for (int i = 0; i < nn; ++i) {
      const size_t sm = (size_t)(rfs[i].P + p->lmax + 1) * sizeof(double2);
      const int cls = sm <= two_per_sm ? 0 : 1;
      if (cls != cls_prev && p->fft_nseg < 8) {
        p->fft_seg_pmin[p->fft_nseg] = rfs[i].P;
        p->fft_seg_gen[p->fft_nseg] = 0;
        long long* sg = p->fft_seg + 3 * p->fft_nseg++;
        sg[0] = i;
        sg[1] = i + 1;
        sg[2] = (long long)sm;
        cls_prev = cls;
      } else {
        long long* sg = p->fft_seg + 3 * (p->fft_nseg - 1);
        sg[1] = i + 1;
        if ((long long)sm > sg[2]) sg[2] = (long long)sm;
        if (rfs[i].P < p->fft_seg_pmin[p->fft_nseg - 1]) p->fft_seg_pmin[p->fft_nseg - 1] = rfs[i].P;
      }
      if (rfs[i].bluestein || rfs[i].r3 || rfs[i].nd != rfs[i].n) p->fft_seg_gen[p->fft_nseg - 1] = 1;
    }
  }
  p->Pmax = lay.Pmax;
  p->Tmax = lay.Tmax;
  p->logTmax = lay.logTmax;
  p->P3max = lay.P3max;
  p->fft_smem = lay.smem;
  p->fft_chirp_total = lay.chirp_total;
  p->fft_bhat_total = lay.bhat_total;
  p->fft_rtw_total = lay.rtw_total;
  FSHT_CUDA_TRY(cudaMalloc(&p->d_rfft, sizeof(FshtRingFFT) * nn));
  FSHT_CUDA_TRY(cudaMemcpyAsync(p->d_rfft, rfs.data(), sizeof(FshtRingFFT) * nn,
                                cudaMemcpyHostToDevice, p->stream));
  const long long ntw = fsht_tw_entries(lay.Tmax, lay.P3max);
  FSHT_CUDA_TRY(cudaMalloc(&p->d_tw, sizeof(double2) * (ntw > 0 ? ntw : 1)));
  FSHT_CUDA_TRY(cudaMalloc(&p->d_chirp, sizeof(double2) * (lay.chirp_total > 0 ? lay.chirp_total : 1)));
  FSHT_CUDA_TRY(cudaMalloc(&p->d_bhat, sizeof(double2) * (lay.bhat_total > 0 ? lay.bhat_total : 1)));
  FSHT_CUDA_TRY(cudaMalloc(&p->d_rtw, sizeof(double2) * (lay.rtw_total > 0 ? lay.rtw_total : 1)));
  int* d_rings = nullptr;
  if (lay.nblue > 0) {
    FSHT_CUDA_TRY(cudaMalloc(&d_rings, sizeof(int) * lay.nblue));
    FSHT_CUDA_TRY(cudaMemcpyAsync(d_rings, blue_rings.data(), sizeof(int) * lay.nblue,
                                  cudaMemcpyHostToDevice, p->stream));
  }
  rc = fsht_fft_tables_fill(p, d_rings, lay.nblue, p->stream);
  FSHT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  if (d_rings) FSHT_CUDA_TRY(cudaFree(d_rings));
  return rc;
}

int fsht_launch_ring_skip(fsht_plan* p, cudaStream_t s) {
  const int lcap = (4 * p->nside > p->lmax) ? 4 * p->nside : p->lmax;
  int* d_first = nullptr;
  FSHT_CUDA_TRY(cudaMalloc(&d_first, sizeof(int) * (p->lmax + 1)));
  k_ring_first_kept<<<(p->lmax + 1 + 63) / 64, 64, 0, s>>>(p->d_cth, p->d_sth, p->d_pref,
                                                             p->nnorth, lcap, p->lmax, d_first);
  FSHT_LAUNCH_CHECK();
  FSHT_CUDA_TRY(cudaMemcpyAsync(p->h_ring_i0, d_first, sizeof(int) * (p->lmax + 1),
                                cudaMemcpyDeviceToHost, s));
  FSHT_CUDA_TRY(cudaStreamSynchronize(s));
  FSHT_CUDA_TRY(cudaFree(d_first));
  int run = 0;
  for (int m = 0; m <= p->lmax; ++m) {
    if (p->h_ring_i0[m] > run) run = p->h_ring_i0[m];
    p->h_ring_i0[m] = run;
  }
  FSHT_CUDA_TRY(cudaMemcpyAsync(p->d_ring_i0, p->h_ring_i0, sizeof(int) * (p->lmax + 1),
                                cudaMemcpyHostToDevice, s));
  FSHT_CUDA_TRY(cudaStreamSynchronize(s));
  return FSHT_OK;
}

int fsht_launch_ring_fft_fwd(fsht_plan* p, const double* maps, long long map_stride, int kc,
                             double2* W, cudaStream_t s) {
  return fsht_launch_ring_fft_fwd_part(p, maps, map_stride, kc, 0, kc, W, s);
}

int fsht_launch_ring_fft_fwd_part(fsht_plan* p, const double* maps, long long map_stride, int kc,
                                  int k0, int kb, double2* W, cudaStream_t s) {
  if (p->d_tw_df) return fsht_launch_ring_fft_fwd_df(p, maps, map_stride, kc, k0, kb, W, s);
  FwdArgs a;
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
  a.tw = plan_tw(p);
  a.rtw = p->d_rtw;
  a.chirp = p->d_chirp;
  a.bhat = p->d_bhat;
  a.ring_i0 = p->d_ring_i0;
  a.W = W;
  a.maps_per_block = p->fft_mpb > 0 ? p->fft_mpb : maps_per_block_for(kb, p->nnorth);
  FSHT_TRY(fsht_smem_limit((const void*)k_ring_fft_fwd, (size_t)(p->fft_smem)));
  for (int sgi = 0; sgi < p->fft_nseg; ++sgi) {
    const long long* sg = p->fft_seg + 3 * sgi;
    a.ring_base = (int)sg[0];
    dim3 grid((unsigned)(sg[1] - sg[0]), (kb + a.maps_per_block - 1) / a.maps_per_block);
    k_ring_fft_fwd<<<grid, p->fft_threads > 0 ? p->fft_threads : 512, (size_t)sg[2], s>>>(a);
    FSHT_LAUNCH_CHECK();
  }
  return FSHT_OK;
}

int fsht_launch_ring_fft_inv(fsht_plan* p, const double2* W, double* maps, long long map_stride,
                             int kc, cudaStream_t s) {
  if (p->d_tw_df) return fsht_launch_ring_fft_inv_df(p, W, maps, map_stride, kc, s);
  InvArgs a;
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
  a.tw = plan_tw(p);
  a.rtw = p->d_rtw;
  a.chirp = p->d_chirp;
  a.bhat = p->d_bhat;
  a.ring_i0 = p->d_ring_i0;
  a.maps_per_block = p->fft_mpb > 0 ? p->fft_mpb : maps_per_block_for(kc, p->nnorth);
  FSHT_TRY(fsht_smem_limit((const void*)k_ring_fft_inv, (size_t)(p->fft_smem)));
  for (int sgi = 0; sgi < p->fft_nseg; ++sgi) {
    const long long* sg = p->fft_seg + 3 * sgi;
    a.ring_base = (int)sg[0];
    dim3 grid((unsigned)(sg[1] - sg[0]), (kc + a.maps_per_block - 1) / a.maps_per_block);
    k_ring_fft_inv<<<grid, p->fft_threads > 0 ? p->fft_threads : 512, (size_t)sg[2], s>>>(a);
    FSHT_LAUNCH_CHECK();
  }
  return FSHT_OK;
}

int fsht_launch_fourier_residual(fsht_plan* p, const double2* X, double2* GR, int kc,
                                 int prefix, cudaStream_t s) {
  ResArgs a;
  a.X = X;
  a.GR = GR;
  a.kc = kc;
  a.nside = p->nside;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.ring_base = 0;
  a.prefix = prefix;
  a.rfs = p->d_rfft;
  a.ring_i0 = p->d_ring_i0;
  a.maps_per_block = p->fft_mpb > 0 ? p->fft_mpb : maps_per_block_for(kc, p->nnorth);
  dim3 grid(p->nnorth, (kc + a.maps_per_block - 1) / a.maps_per_block);
  FSHT_TRY(fsht_smem_limit((const void*)k_fourier_residual, (size_t)(p->fft_smem)));
  k_fourier_residual<<<grid, p->fft_threads > 0 ? p->fft_threads : 512, p->fft_smem, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}
