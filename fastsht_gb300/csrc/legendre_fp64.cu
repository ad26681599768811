// FP64 Legendre contraction (the plain method) with the associated-Legendre
// recursion computed on the fly, north/south folded by l+m parity.
//
// Replaces, per order m, the reference's get_plm_recursive
// (src/get_plm_recursive.f90:17-136) + mat2alm / alm2mat DGEMMs
// (src/sht_core.f90:30-168).  No P_lm table is materialised: each CTA carries the
// recursion state of its rings in shared memory (analysis) or registers
// (synthesis) and produces lambda tiles just before they are consumed.
//
// Recursion (get_plm_recursive.f90:31-67):
//   lambda_mm = sqrt(diag_fac(m)/(4 pi)) (-sin theta)^m,
//   lambda_l  = a_l cos(theta) lambda_{l-1} - b_l lambda_{l-2},
//   a_l = sqrt((4l^2-1)/(l^2-m^2)),  b_l = sqrt(((l-1)^2-m^2)/(4(l-1)^2-1)) a_l.
// Values are carried as v * 2^(600 e) with an integer e <= 0 per ring, so polar
// rings at large m never underflow (this replaces the reference's nside > 512
// "safe start" tables, plm_table/*.bin); while e < 0 the true value is below
// 2^-300 and the tile gets 0.
//
// FP64 on GB300 runs at ~1.2 TFLOP/s (DFMA) and its DMMA (mma.sync f64) is no
// faster, so these kernels are plain register-tiled DFMA: every thread keeps an
// accumulator tile in registers and reads shared-memory tiles laid out so that a
// warp's loads are conflict-free.
#include "common.cuh"

namespace {

constexpr int LC = 32;    // l values per chunk (even: keeps l-m parity static per slot)
constexpr int NT = 256;   // threads per CTA

struct RecConst {         // per (m, l) coefficients
  double a, b;
};

__device__ __forceinline__ RecConst rec_coeffs(int l, int m) {
  RecConst c;
  const long long L = l, M = m;
  // c3/(c4 - m^2) and (c1 - m^2)/c2 with exact integer numerators/denominators
  // (set_out_of_loop_constants, src/sht_data_init.f90:405-409)
  c.a = sqrt((double)((2 * L - 1) * (2 * L + 1)) / (double)(L * L - M * M));
  c.b = sqrt((double)((L - 1) * (L - 1) - M * M) / (double)((2 * L - 3) * (2 * L - 1))) * c.a;
  return c;
}

// lambda_mm in the scaled representation: value = cur * 2^(600 e).
__device__ __forceinline__ void rec_seed(double sth, double pref, int m, double& cur, int& e) {
  int ex;
  double mt = frexp(sth, &ex);
  double rm = 1.0, bm = mt;
  long long re = 0, be = ex;
  for (int k = m; k; k >>= 1) {
    if (k & 1) { rm *= bm; re += be; int t; rm = frexp(rm, &t); re += t; }
    if (k > 1) { bm *= bm; be *= 2; int t; bm = frexp(bm, &t); be += t; }
  }
  rm *= pref;
  { int t; rm = frexp(rm, &t); re += t; }
  if (m & 1) rm = -rm;
  e = (re >= -300) ? 0 : (int)floor((double)(re + 300) / 600.0);
  cur = ldexp(rm, (int)(re - 600LL * e));
}

__device__ __forceinline__ void rec_step(double& cur, double& prev, int& e, double a_cth,
                                         double b) {
  const double nx = a_cth * cur - b * prev;
  prev = cur;
  cur = nx;
  if (e < 0 && fabs(cur) > 0x1p300) {
    cur *= 0x1p-600;
    prev *= 0x1p-600;
    ++e;
  }
}

// Spin-2 lambda1/lambda2 from lambda_l (cur) and lambda_{l-1} (prev) on one ring
// (get_plm_recursive.f90:101-125).
struct PolRing {
  double cth, b_w, two_on_s2, c_w, diag1, diag2;
};
__device__ __forceinline__ PolRing pol_ring(double cth, double sth, int m) {
  PolRing r;
  const double s2 = sth * sth;
  r.cth = cth;
  r.b_w = cth / s2;
  r.two_on_s2 = 2.0 / s2;
  r.c_w = (double)m / s2;
  r.diag1 = 0.5 - 1.0 / s2;
  r.diag2 = cth / s2;
  return r;
}
__device__ __forceinline__ double normal_l(int l) {
  if (l < 2) return 0.0;
  return 1.0 / sqrt((double)(l + 2) * (double)(l + 1) * (double)l * (double)(l - 1));
}
__device__ __forceinline__ double lam_fact(int l, int m) {
  const int m1 = m > 1 ? m : 1;
  if (l <= m1) return 0.0;
  return 2.0 * sqrt((double)(2 * l + 1) / (double)(2 * l - 1) * (double)((long long)l * l - (long long)m * m));
}
__device__ __forceinline__ void pol_lambda(const PolRing& r, int l, int m, double cur, double prev,
                                           double lf, double nl, double& l1, double& l2) {
  if (l == m) {
    const double nm = (double)(2LL * m * (1 - m)) * nl;
    l1 = nm * cur * r.diag1;
    l2 = nm * cur * r.diag2;
  } else {
    l1 = (prev * lf * r.b_w - cur * (r.two_on_s2 * (double)((long long)l - (long long)m * m) +
                                     (double)l * ((double)l - 1.0))) * nl;
    l2 = (prev * lf - cur * (2.0 * r.cth * ((double)l - 1.0))) * r.c_w * nl;
  }
}

// ====================================================================== analysis
struct AnaArgs {
  int nside, lmax, nnorth;
  const double* cth;
  const double* sth;
  const double* pref;
  const int* ring_i0;
  const double2* WQ;   // {S, D} per (m, ring, map); T or Q
  const double2* WU;   // U (spin 2)
  int kc;              // maps in the chunk (W's map extent)
  double* almE;        // T or E
  double* almB;
  int ld;              // alm map extent (total nmaps)
  int k0;              // alm map offset of this chunk
  double scale;        // pa (T) or -pa (spin 2)
  int accumulate;
  int which;           // bit0: E/T, bit1: B
};

// Tile shape: QN map slots per thread (16 QN maps per CTA: 64 by default, 32 for small
// batches) and RC rings per chunk (16 for spin 0 and 8 for spin 2 by default); the autotuner
// picks among the instantiated shapes per (nside, lmax) bucket.
template <int SPIN, int QN = 4, int RCN = (SPIN == 0 ? 16 : 8)>
struct AnaCfg {
  static constexpr int MT = 16 * QN;             // maps per CTA
  static constexpr int RC = RCN;                 // rings per chunk
  static constexpr int NF = SPIN == 0 ? 1 : 2;   // fields read
};

template <int SPIN, int QN, int RCN>
__global__ void __launch_bounds__(NT) k_analysis_fp64(AnaArgs a) {
  using C = AnaCfg<SPIN, QN, RCN>;
  constexpr int MT = C::MT, RC = C::RC, NF = C::NF;
  extern __shared__ __align__(16) double smem_d[];
  // layout: st_cur[nnorth] st_prev[nnorth] | P[NF][2][RC][MT] double2 | lam1[RC][LC]
  //         (lam2[RC][LC]) | st_e[nnorth] int
  double* st_cur = smem_d;
  double* st_prev = st_cur + a.nnorth;
  double2* P = reinterpret_cast<double2*>(st_prev + a.nnorth);
  double* lam1 = reinterpret_cast<double*>(P + NF * 2 * RC * MT);
  double* lam2 = lam1 + RC * LC;
  int* st_e = reinterpret_cast<int*>(lam2 + (SPIN == 2 ? RC * LC : 0));
  __shared__ double s_lf[LC], s_nl[LC];
  __shared__ RecConst s_rc[LC];

  const int tid = threadIdx.x;
  const int mg = tid & 15;        // maps mg + 16 q
  const int lg = tid >> 4;        // l slots lg, lg + 16 (same l-m parity)
  const int par = lg & 1;
  const int kt0 = blockIdx.y * MT;
  const int npair = (a.lmax + 2) / 2;
  // map slots q with a map behind them: small batches skip the padding's FMAs (warps
  // whose lanes all lack slot q skip it entirely)
  const int nq = max(0, min(QN, (a.kc - kt0 - mg + 15) / 16));

  for (int pass = 0; pass < 2; ++pass) {
    const int m = pass == 0 ? (int)blockIdx.x : a.lmax - (int)blockIdx.x;
    if (pass == 1 && m == (int)blockIdx.x) break;
    if (m < 0) break;
    (void)npair;
    const int i0 = a.ring_i0[m];
    const int nr = a.nnorth - i0;
    __syncthreads();
    for (int r = tid; r < nr; r += NT) {
      double cur;
      int e;
      rec_seed(a.sth[i0 + r], a.pref[m], m, cur, e);
      st_cur[r] = cur;
      st_prev[r] = 0.0;
      st_e[r] = e;
    }
    for (int l0 = m; l0 <= a.lmax; l0 += LC) {
      const int nl = min(LC, a.lmax + 1 - l0);
      if (tid < LC) {
        const int l = l0 + tid;
        RecConst rc{0.0, 0.0};
        if (l > m && l <= a.lmax) rc = rec_coeffs(l, m);
        s_rc[tid] = rc;
        if (SPIN == 2) {
          s_lf[tid] = (l <= a.lmax) ? lam_fact(l, m) : 0.0;
          s_nl[tid] = (l <= a.lmax) ? normal_l(l) : 0.0;
        }
      }
      double2 accE[2][QN], accB[2][QN];
#pragma unroll
      for (int s = 0; s < 2; ++s)
#pragma unroll
        for (int q = 0; q < QN; ++q) {
          accE[s][q] = make_double2(0.0, 0.0);
          accB[s][q] = make_double2(0.0, 0.0);
        }
      for (int r0 = 0; r0 < nr; r0 += RC) {
        __syncthreads();
        // ---- lambda tile (RC threads, one ring each)
        if (tid < RC) {
          const int r = r0 + tid;
          if (r < nr) {
            double cur = st_cur[r], prev = st_prev[r];
            int e = st_e[r];
            const int ir = i0 + r;
            const double cth = a.cth[ir];
            PolRing pr;
            if (SPIN == 2) pr = pol_ring(cth, a.sth[ir], m);
            for (int j = 0; j < LC; ++j) {
              const int l = l0 + j;
              if (j < nl && l > m) rec_step(cur, prev, e, s_rc[j].a * cth, s_rc[j].b);
              const bool ok = (j < nl) && (e == 0);
              if (SPIN == 0) {
                lam1[tid * LC + j] = ok ? cur : 0.0;
              } else {
                double l1 = 0.0, l2 = 0.0;
                if (ok) pol_lambda(pr, l, m, cur, prev, s_lf[j], s_nl[j], l1, l2);
                lam1[tid * LC + j] = l1;
                lam2[tid * LC + j] = l2;
              }
            }
            st_cur[r] = cur;
            st_prev[r] = prev;
            st_e[r] = e;
          } else {
            for (int j = 0; j < LC; ++j) {
              lam1[tid * LC + j] = 0.0;
              if (SPIN == 2) lam2[tid * LC + j] = 0.0;
            }
          }
        }
        // ---- phase tile P[f][s][rr][map] from W[m][i0+r0+rr][kt0+map][s]
        for (int idx = tid; idx < NF * 2 * RC * MT; idx += NT) {
          const int map = idx % MT;
          const int s = (idx / MT) & 1;
          const int rr = (idx / (2 * MT)) % RC;
          const int f = idx / (2 * MT * RC);
          const int r = r0 + rr;
          const int k = kt0 + map;
          double2 v = make_double2(0.0, 0.0);
          if (r < nr && k < a.kc) {
            const double2* W = (f == 0) ? a.WQ : a.WU;
            v = W[(((long long)m * a.nnorth + i0 + r) * a.kc + k) * 2 + s];
          }
          P[((f * 2 + s) * RC + rr) * MT + map] = v;
        }
        __syncthreads();
        const int nrr = min(RC, nr - r0);
        for (int rr = 0; rr < nrr; ++rr) {
          if (SPIN == 0) {
            const double la = lam1[rr * LC + lg];
            const double lb = lam1[rr * LC + lg + 16];
            const double2* pp = P + (par * RC + rr) * MT + mg;
#pragma unroll
            for (int q = 0; q < QN; ++q) {
              if (q >= nq) break;
              const double2 v = pp[16 * q];
              accE[0][q].x = fma(la, v.x, accE[0][q].x);
              accE[0][q].y = fma(la, v.y, accE[0][q].y);
              accE[1][q].x = fma(lb, v.x, accE[1][q].x);
              accE[1][q].y = fma(lb, v.y, accE[1][q].y);
            }
          } else {
            const double l1a = lam1[rr * LC + lg], l1b = lam1[rr * LC + lg + 16];
            const double l2a = lam2[rr * LC + lg], l2b = lam2[rr * LC + lg + 16];
            // P1 = S for even l-m, D for odd; P2 the other one
            const double2* q1 = P + ((0 * 2 + par) * RC + rr) * MT + mg;
            const double2* q2 = P + ((0 * 2 + (1 - par)) * RC + rr) * MT + mg;
            const double2* u1 = P + ((1 * 2 + par) * RC + rr) * MT + mg;
            const double2* u2 = P + ((1 * 2 + (1 - par)) * RC + rr) * MT + mg;
#pragma unroll
            for (int q = 0; q < QN; ++q) {
              if (q >= nq) break;
              const double2 Q1 = q1[16 * q], Q2 = q2[16 * q], U1 = u1[16 * q], U2 = u2[16 * q];
              // E += l1 P1Q + i l2 P2U ;  B += l1 P1U - i l2 P2Q
              accE[0][q].x = fma(l1a, Q1.x, fma(-l2a, U2.y, accE[0][q].x));
              accE[0][q].y = fma(l1a, Q1.y, fma(l2a, U2.x, accE[0][q].y));
              accE[1][q].x = fma(l1b, Q1.x, fma(-l2b, U2.y, accE[1][q].x));
              accE[1][q].y = fma(l1b, Q1.y, fma(l2b, U2.x, accE[1][q].y));
              accB[0][q].x = fma(l1a, U1.x, fma(l2a, Q2.y, accB[0][q].x));
              accB[0][q].y = fma(l1a, U1.y, fma(-l2a, Q2.x, accB[0][q].y));
              accB[1][q].x = fma(l1b, U1.x, fma(l2b, Q2.y, accB[1][q].x));
              accB[1][q].y = fma(l1b, U1.y, fma(-l2b, Q2.x, accB[1][q].y));
            }
          }
        }
      }
      // ---- epilogue: square-real alm, Re at [m][l][k], Im at [lmax+1-m][l-m][k]
      const long long L1 = a.lmax + 1;
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const int j = lg + 16 * s;
        const int l = l0 + j;
        if (j >= nl) continue;
#pragma unroll
        for (int q = 0; q < QN; ++q) {
          const int k = kt0 + mg + 16 * q;
          if (k >= a.kc) continue;
          const long long kk = a.k0 + k;
          const long long re_idx = ((long long)m * L1 + l) * a.ld + kk;
          const long long im_idx = ((L1 - m) * L1 + (l - m)) * a.ld + kk;
          for (int fld = 0; fld < (SPIN == 0 ? 1 : 2); ++fld) {
            if (!(a.which & (1 << fld))) continue;
            double* alm = fld == 0 ? a.almE : a.almB;
            const double2 v = cscale(fld == 0 ? accE[s][q] : accB[s][q], a.scale);
            if (a.accumulate) {
              alm[re_idx] += v.x;
              if (m > 0) alm[im_idx] += v.y;
            } else {
              alm[re_idx] = v.x;
              if (m > 0) alm[im_idx] = v.y;
            }
          }
        }
      }
    }
  }
}

// ====================================================================== synthesis
struct SynArgs {
  int nside, lmax, nnorth;
  const double* cth;
  const double* sth;
  const double* pref;
  const int* ring_i0;
  const double* almE;   // T or E
  const double* almB;
  int ld, k0;
  double2* WQ;          // {G_N, G_S} per (m, ring, map); T or Q
  double2* WU;
  int kc;
};

template <int SPIN>
struct SynCfg {
  static constexpr int MQ = SPIN == 0 ? 4 : 2;   // maps per thread
  static constexpr int MT = 16 * MQ;             // maps per CTA
  static constexpr int RCS = 32;                 // rings per CTA
};

template <int SPIN>
__global__ void __launch_bounds__(NT) k_synthesis_fp64(SynArgs a) {
  using C = SynCfg<SPIN>;
  constexpr int MQ = C::MQ, MT = C::MT, RCS = C::RCS;
  constexpr int NF = SPIN == 0 ? 1 : 2;
  extern __shared__ __align__(16) double2 smem_s[];
  // dynamic layout: A[NF][LC][MT] (alm tile) | lam1[RCS][LC+1] | lam2[RCS][LC+1]
  auto A = reinterpret_cast<double2(*)[LC][MT]>(smem_s);
  auto lam1 = reinterpret_cast<double(*)[LC + 1]>(smem_s + NF * LC * MT);
  auto lam2 = reinterpret_cast<double(*)[LC + 1]>(smem_s + NF * LC * MT) + RCS;
  __shared__ RecConst s_rc[LC];
  __shared__ double s_lf[LC], s_nl[LC];

  const int tid = threadIdx.x;
  const int mg = tid & 15;   // maps mg + 16 q
  const int rg = tid >> 4;   // rings rg, rg + 16 of the chunk
  const int ib = blockIdx.y * RCS;
  const int kt0 = blockIdx.z * MT;
  const long long L1 = a.lmax + 1;
  const int nq = max(0, min(MQ, (a.kc - kt0 - mg + 15) / 16));   // map slots with a map

  for (int pass = 0; pass < 2; ++pass) {
    const int m = pass == 0 ? (int)blockIdx.x : a.lmax - (int)blockIdx.x;
    if (pass == 1 && m == (int)blockIdx.x) break;
    const int i0 = a.ring_i0[m];
    if (ib + RCS <= i0) continue;          // no ring of this chunk is kept for m
    // recursion state for ring ib + tid (warp 0)
    double cur = 0.0, prev = 0.0;
    int e = -1;
    double cth = 0.0;
    PolRing pr;
    const int ir = ib + tid;
    const bool rown = tid < RCS && ir >= i0 && ir < a.nnorth;
    if (rown) {
      cth = a.cth[ir];
      rec_seed(a.sth[ir], a.pref[m], m, cur, e);
      if (SPIN == 2) pr = pol_ring(cth, a.sth[ir], m);
    }
    // accumulators [parity][field-product][q][ring] (complex)
    constexpr int NP = SPIN == 0 ? 1 : 4;
    double2 acc[2][NP][MQ][2];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int t = 0; t < NP; ++t)
#pragma unroll
        for (int q = 0; q < MQ; ++q) {
          acc[s][t][q][0] = make_double2(0.0, 0.0);
          acc[s][t][q][1] = make_double2(0.0, 0.0);
        }
    for (int l0 = m; l0 <= a.lmax; l0 += LC) {
      const int nl = min(LC, a.lmax + 1 - l0);
      __syncthreads();
      if (tid < LC) {
        const int l = l0 + tid;
        RecConst rc{0.0, 0.0};
        if (l > m && l <= a.lmax) rc = rec_coeffs(l, m);
        s_rc[tid] = rc;
        if (SPIN == 2) {
          s_lf[tid] = (l <= a.lmax) ? lam_fact(l, m) : 0.0;
          s_nl[tid] = (l <= a.lmax) ? normal_l(l) : 0.0;
        }
      }
      // alm tile
      for (int idx = tid; idx < NF * LC * MT; idx += NT) {
        const int map = idx % MT;
        const int j = (idx / MT) % LC;
        const int f = idx / (MT * LC);
        const int l = l0 + j;
        const int k = kt0 + map;
        double2 v = make_double2(0.0, 0.0);
        if (j < nl && k < a.kc) {
          const double* alm = f == 0 ? a.almE : a.almB;
          const long long kk = a.k0 + k;
          v.x = alm[((long long)m * L1 + l) * a.ld + kk];
          if (m > 0) v.y = alm[((L1 - m) * L1 + (l - m)) * a.ld + kk];
        }
        A[f][j][map] = v;
      }
      __syncthreads();
      if (tid < RCS) {
        for (int j = 0; j < LC; ++j) {
          const int l = l0 + j;
          if (rown && j < nl && l > m) rec_step(cur, prev, e, s_rc[j].a * cth, s_rc[j].b);
          const bool ok = rown && (j < nl) && (e == 0);
          if (SPIN == 0) {
            lam1[tid][j] = ok ? cur : 0.0;
          } else {
            double l1 = 0.0, l2 = 0.0;
            if (ok) pol_lambda(pr, l, m, cur, prev, s_lf[j], s_nl[j], l1, l2);
            lam1[tid][j] = l1;
            lam2[tid][j] = l2;
          }
        }
      }
      __syncthreads();
#pragma unroll 2
      for (int j = 0; j < LC; j += 2) {
#pragma unroll
        for (int s = 0; s < 2; ++s) {      // s = parity of l - m (l0 - m is even)
          const int jj = j + s;
          if (SPIN == 0) {
            const double r0 = lam1[rg][jj], r1 = lam1[rg + 16][jj];
#pragma unroll
            for (int q = 0; q < MQ; ++q) {
              if (q >= nq) break;
              const double2 v = A[0][jj][mg + 16 * q];
              acc[s][0][q][0].x = fma(r0, v.x, acc[s][0][q][0].x);
              acc[s][0][q][0].y = fma(r0, v.y, acc[s][0][q][0].y);
              acc[s][0][q][1].x = fma(r1, v.x, acc[s][0][q][1].x);
              acc[s][0][q][1].y = fma(r1, v.y, acc[s][0][q][1].y);
            }
          } else {
            const double a10 = lam1[rg][jj], a11 = lam1[rg + 16][jj];
            const double a20 = lam2[rg][jj], a21 = lam2[rg + 16][jj];
#pragma unroll
            for (int q = 0; q < MQ; ++q) {
              if (q >= nq) break;
              const double2 E = A[0][jj][mg + 16 * q];
              const double2 B = A[1][jj][mg + 16 * q];
              // t=0: l1 E, t=1: l2 B, t=2: l2 E, t=3: l1 B
              acc[s][0][q][0].x = fma(a10, E.x, acc[s][0][q][0].x);
              acc[s][0][q][0].y = fma(a10, E.y, acc[s][0][q][0].y);
              acc[s][0][q][1].x = fma(a11, E.x, acc[s][0][q][1].x);
              acc[s][0][q][1].y = fma(a11, E.y, acc[s][0][q][1].y);
              acc[s][1][q][0].x = fma(a20, B.x, acc[s][1][q][0].x);
              acc[s][1][q][0].y = fma(a20, B.y, acc[s][1][q][0].y);
              acc[s][1][q][1].x = fma(a21, B.x, acc[s][1][q][1].x);
              acc[s][1][q][1].y = fma(a21, B.y, acc[s][1][q][1].y);
              acc[s][2][q][0].x = fma(a20, E.x, acc[s][2][q][0].x);
              acc[s][2][q][0].y = fma(a20, E.y, acc[s][2][q][0].y);
              acc[s][2][q][1].x = fma(a21, E.x, acc[s][2][q][1].x);
              acc[s][2][q][1].y = fma(a21, E.y, acc[s][2][q][1].y);
              acc[s][3][q][0].x = fma(a10, B.x, acc[s][3][q][0].x);
              acc[s][3][q][0].y = fma(a10, B.y, acc[s][3][q][0].y);
              acc[s][3][q][1].x = fma(a11, B.x, acc[s][3][q][1].x);
              acc[s][3][q][1].y = fma(a11, B.y, acc[s][3][q][1].y);
            }
          }
        }
      }
    }
    // ---- epilogue: north = even + odd, south = even - odd (lambda_S = (-1)^(l-m) lambda_N)
#pragma unroll
    for (int rsel = 0; rsel < 2; ++rsel) {
      const int i = ib + rg + 16 * rsel;
      if (i < i0 || i >= a.nnorth) continue;
#pragma unroll
      for (int q = 0; q < MQ; ++q) {
        const int k = kt0 + mg + 16 * q;
        if (k >= a.kc) continue;
        const long long w = (((long long)m * a.nnorth + i) * a.kc + k) * 2;
        if (SPIN == 0) {
          const double2 ev = acc[0][0][q][rsel], od = acc[1][0][q][rsel];
          a.WQ[w] = cadd(ev, od);
          a.WQ[w + 1] = csub(ev, od);
        } else {
          // lambda1_S = s lambda1_N, lambda2_S = -s lambda2_N, s = (-1)^(l-m)
          const double2 X1e = acc[0][0][q][rsel], X1o = acc[1][0][q][rsel];   // l1 E
          const double2 Y2e = acc[0][1][q][rsel], Y2o = acc[1][1][q][rsel];   // l2 B
          const double2 X2e = acc[0][2][q][rsel], X2o = acc[1][2][q][rsel];   // l2 E
          const double2 Y1e = acc[0][3][q][rsel], Y1o = acc[1][3][q][rsel];   // l1 B
          const double2 x1n = cadd(X1e, X1o), x1s = csub(X1e, X1o);
          const double2 y2n = cadd(Y2e, Y2o), y2s = csub(Y2o, Y2e);
          const double2 x2n = cadd(X2e, X2o), x2s = csub(X2o, X2e);
          const double2 y1n = cadd(Y1e, Y1o), y1s = csub(Y1e, Y1o);
          // G_Q = -(l1 E + i l2 B);  G_U = i l2 E - l1 B
          a.WQ[w] = make_double2(-x1n.x + y2n.y, -x1n.y - y2n.x);
          a.WQ[w + 1] = make_double2(-x1s.x + y2s.y, -x1s.y - y2s.x);
          a.WU[w] = make_double2(-x2n.y - y1n.x, x2n.x - y1n.y);
          a.WU[w + 1] = make_double2(-x2s.y - y1s.x, x2s.x - y1s.y);
        }
      }
    }
  }
}

template <int SPIN>
size_t syn_smem() {
  using C = SynCfg<SPIN>;
  constexpr int NF = SPIN == 0 ? 1 : 2;
  return sizeof(double2) * NF * LC * C::MT + sizeof(double) * C::RCS * (LC + 1) * (SPIN == 2 ? 2 : 1);
}

template <int SPIN, int QN, int RCN>
size_t ana_smem(int nnorth) {
  using C = AnaCfg<SPIN, QN, RCN>;
  return (size_t)nnorth * (2 * sizeof(double) + sizeof(int)) +
         sizeof(double2) * C::NF * 2 * C::RC * C::MT +
         sizeof(double) * C::RC * LC * (SPIN == 2 ? 2 : 1);
}

template <int SPIN, int QN, int RCN>
int launch_ana(const AnaArgs& a, int npair, int nnorth, int kc, cudaStream_t s) {
  using C = AnaCfg<SPIN, QN, RCN>;
  const size_t sm = ana_smem<SPIN, QN, RCN>(nnorth);
  FSHT_TRY(fsht_smem_limit((const void*)k_analysis_fp64<SPIN, QN, RCN>, sm));
  dim3 grid(npair, (kc + C::MT - 1) / C::MT);
  k_analysis_fp64<SPIN, QN, RCN><<<grid, NT, sm, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

}  // namespace

int fsht_launch_analysis_fp64(fsht_plan* p, int spin, const double2* WQ, const double2* WU,
                              double* almE, double* almB, int nmaps_total, int k0, int kc,
                              int accumulate, int which, cudaStream_t s) {
  AnaArgs a;
  a.nside = p->nside;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.cth = p->d_cth;
  a.sth = p->d_sth;
  a.pref = p->d_pref;
  a.ring_i0 = p->d_ring_i0;
  a.WQ = WQ;
  a.WU = WU;
  a.kc = kc;
  a.almE = almE;
  a.almB = almB;
  a.ld = nmaps_total;
  a.k0 = k0;
  a.scale = spin == 0 ? p->pa : -p->pa;
  a.accumulate = accumulate;
  a.which = which;
  const int npair = (p->lmax + 2) / 2;
  // tile shape: the plan's (autotuned) choice, else the default 64 maps per CTA
  const bool q2 = p->ana_mt == 32;
  if (spin == 0) {
    if (p->ana_rc == 32)
      return q2 ? launch_ana<0, 2, 32>(a, npair, p->nnorth, kc, s)
                : launch_ana<0, 4, 32>(a, npair, p->nnorth, kc, s);
    if (p->ana_rc == 8)
      return q2 ? launch_ana<0, 2, 8>(a, npair, p->nnorth, kc, s)
                : launch_ana<0, 4, 8>(a, npair, p->nnorth, kc, s);
    return q2 ? launch_ana<0, 2, 16>(a, npair, p->nnorth, kc, s)
              : launch_ana<0, 4, 16>(a, npair, p->nnorth, kc, s);
  }
  if (p->ana_rc == 16)
    return q2 ? launch_ana<2, 2, 16>(a, npair, p->nnorth, kc, s)
              : launch_ana<2, 4, 16>(a, npair, p->nnorth, kc, s);
  return q2 ? launch_ana<2, 2, 8>(a, npair, p->nnorth, kc, s)
            : launch_ana<2, 4, 8>(a, npair, p->nnorth, kc, s);
}

int fsht_launch_synthesis_fp64(fsht_plan* p, int spin, const double* almE, const double* almB,
                               double2* WQ, double2* WU, int nmaps_total, int k0, int kc,
                               cudaStream_t s) {
  SynArgs a;
  a.nside = p->nside;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.cth = p->d_cth;
  a.sth = p->d_sth;
  a.pref = p->d_pref;
  a.ring_i0 = p->d_ring_i0;
  a.almE = almE;
  a.almB = almB;
  a.ld = nmaps_total;
  a.k0 = k0;
  a.WQ = WQ;
  a.WU = WU;
  a.kc = kc;
  const int npair = (p->lmax + 2) / 2;
  if (spin == 0) {
    const size_t sm = syn_smem<0>();
    FSHT_TRY(fsht_smem_limit((const void*)k_synthesis_fp64<0>, (size_t)(sm)));
    dim3 grid(npair, (p->nnorth + SynCfg<0>::RCS - 1) / SynCfg<0>::RCS,
              (kc + SynCfg<0>::MT - 1) / SynCfg<0>::MT);
    k_synthesis_fp64<0><<<grid, NT, sm, s>>>(a);
  } else {
    const size_t sm = syn_smem<2>();
    FSHT_TRY(fsht_smem_limit((const void*)k_synthesis_fp64<2>, (size_t)(sm)));
    dim3 grid(npair, (p->nnorth + SynCfg<2>::RCS - 1) / SynCfg<2>::RCS,
              (kc + SynCfg<2>::MT - 1) / SynCfg<2>::MT);
    k_synthesis_fp64<2><<<grid, NT, sm, s>>>(a);
  }
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}
