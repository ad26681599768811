// Split-precision spin-2 analysis (Q/U -> E/B) on the tcgen05 tensor cores.
//
// The precision form of the reference's QU2EB contraction (get_plm_recursive.f90:101-125 for
// lambda1/lambda2, sht_core.f90:30-89 with the spin-2 GEMM types, sht_main.f90:383-436):
//   E = -pa [ sum_i lambda1 Q_p(i) + i sum_i lambda2 U_{1-p}(i) ]
//   B = -pa [ sum_i lambda1 U_p(i) - i sum_i lambda2 Q_{1-p}(i) ]
// with p = (l - m) mod 2 selecting S (p = 0) or D (p = 1) of each field (lambda1 has the
// north/south parity of lambda, lambda2 the opposite one).  Digits, levels and scales are
// those of the spin-0 form (legendre_split.cu); |lambda1|, |lambda2| <= 0.62 sqrt((2l+1)/4pi)
// (checked against the oracle), so they share the spin-0 row scales.
//
//   k_pol_table          per (l, m): c1..c4 of the scaled lambda1/lambda2 formulas;
//   k_lambda_digits_pol  the df64 recursion (mu form) once per (m, ring), lambda1 and
//                        lambda2 digit tiles into the wave's staging buffer;
//   k_split_gemm_pol     persistent; unit = (q, l-tile, parity, field, 64-map group): per
//                        ring part the lambda1 product then the lambda2 product through the
//                        same TMEM accumulators, each with its own column scales; the
//                        epilogue routes (Re, Im) of the second product by the factor +-i.
// and the spin-2 synthesis (k_lambda_digits_T_pol, k_split_synth_pol) below.
#include "split_common.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

__device__ __forceinline__ double pol_normal_l(int l) {
  if (l < 2) return 0.0;
  return 1.0 / sqrt((double)(l + 2) * (double)(l + 1) * (double)l * (double)(l - 1));
}

// lambda1 / D_l = mu_{l-1} c1 cos/s^2 - mu_l (c2 / s^2 + c3)
// lambda2 / D_l = (mu_{l-1} c1 - mu_l c4 cos) m / s^2
// c1 = lam_fact nl / a_l, c2 = 2 (l - m^2) nl, c3 = l (l - 1) nl, c4 = 2 (l - 1) nl.  At l = m
// (mu_{m-1} = 0) these reduce to the reference's diagonal formulas.
__global__ void k_pol_table(int lmax, FshtPolRow* tab) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m > lmax) return;
  FshtPolRow* row = tab + tri_off(m, lmax);
  const int m1 = m > 1 ? m : 1;
  for (int l = m; l <= lmax; ++l) {
    const double nl = pol_normal_l(l);
    double c1 = 0.0;
    if (l > m && l > m1) {
      const double lf =
          2.0 * sqrt((double)(2 * l + 1) / (double)(2 * l - 1) * (double)((long long)l * l - (long long)m * m));
      c1 = lf * nl / rec_coeffs(l, m).a;
    }
    FshtPolRow r;
    r.c1 = c1;
    r.c2 = 2.0 * ((double)l - (double)m * (double)m) * nl;
    r.c3 = (double)l * ((double)l - 1.0) * nl;
    r.c4 = 2.0 * ((double)l - 1.0) * nl;
    row[l - m] = r;
  }
}

// grid (q in wave, 128-ring block), 128 threads = rings.  Tiles of m: (parity, l-tile,
// part (lambda1, lambda2), k-step) x 4 digits, at twice the spin-0 offset of q.
struct LamPArgs {
  int lmax, nnorth, q0;
  const double* cth;
  const double* sth;
  const double* pref;
  const int* ring_i0;
  const FshtLamRow* tab;
  const FshtPolRow* ptab;
  const long long* lam_off;
  unsigned char* lbuf;
  int* err;
};

constexpr int kPolBlock = 32;                 // l per staging block
constexpr int kPolStride = kSCRings + 2;      // uint64 per staged row (+16 B)
constexpr size_t kPolStageBytes = (size_t)2 * 2 * (kPolBlock / 2) * kPolStride * 8;

__global__ void __launch_bounds__(128) k_lambda_digits_pol(LamPArgs a) {
  extern __shared__ __align__(16) unsigned long long S[];     // [part][parity][row][ring]
  // per staged l: -beta, c1, c2, c3, c4 as df64 pairs
  __shared__ float2 s_beta[kPolBlock];
  __shared__ int s_erow[kPolBlock];
  __shared__ float2 s_pc[kPolBlock][4];
  const int q = a.q0 + blockIdx.x;
  const int m = m_of_q(q, a.lmax);
  const int i0 = a.ring_i0[m];
  const int K = a.nnorth - i0;
  const int rb = blockIdx.y;
  if (rb * kSCRings >= K) return;
  const int tid = threadIdx.x;
  const int r = rb * kSCRings + tid;
  const bool valid = r < K;
  const int nks = (K + kKStep - 1) / kKStep;
  const int ntiles = (a.lmax - m + 1 + 2 * kRows - 1) / (2 * kRows);
  unsigned char* base =
      a.lbuf + (size_t)(2 * (a.lam_off[q] - a.lam_off[a.q0])) * kSlices * kATileBytes;
  const FshtLamRow* tab = a.tab + tri_off(m, a.lmax);
  const FshtPolRow* ptab = a.ptab + tri_off(m, a.lmax);
  auto pair = [](double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
  };
  auto stage = [&](int j0) {
    if (tid < kPolBlock && m + j0 + tid <= a.lmax) {
      s_beta[tid] = pair(-tab[j0 + tid].beta);
      s_erow[tid] = tab[j0 + tid].erow;
      const FshtPolRow c = ptab[j0 + tid];
      s_pc[tid][0] = pair(c.c1);
      s_pc[tid][1] = pair(c.c2);
      s_pc[tid][2] = pair(c.c3);
      s_pc[tid][3] = pair(c.c4);
    }
  };

  // The recursion and the lambda1 / lambda2 forms run in df64 on the FP32 pipe (about 80 FP32
  // instructions per step against ten FP64 operations, which GB300 runs at two per clock per
  // SM); the state is rescaled after every step as in k_lambda_digits.
  float2 x = make_float2(0.f, 0.f), is2 = x, bw = x, cw = x, s1 = x, s2 = x;
  int et = 0;
  if (valid) {
    int e, kx;
    const double sth = a.sth[i0 + r];
    const double xd = a.cth[i0 + r];
    const double inv_s2 = 1.0 / (sth * sth);
    double sd;
    rec_seed(sth, a.pref[m], m, sd, e);
    const double f = frexp(sd, &kx);
    et = 600 * e + kx;
    s1 = pair(f);
    x = pair(xd);
    is2 = pair(inv_s2);
    bw = pair(xd * inv_s2);
    cw = pair((double)m * inv_s2);
  }
  stage(0);
  __syncthreads();
  const int lend = ntiles * 2 * kRows;
  auto Sidx = [&](int part, int par, int row, int col) -> unsigned long long& {
    return S[((part * 2 + par) * (kPolBlock / 2) + row) * kPolStride + col];
  };
  bool bad = false;
  for (int lb = 0; lb < lend; lb += kPolBlock) {
#pragma unroll 2
    for (int jj = 0; jj < kPolBlock; ++jj) {
      const int j = lb + jj;
      unsigned long long pk1 = 0, pk2 = 0;
      if (m + j <= a.lmax) {
        if (j > 0) {
          const float2 nb = s_beta[jj];
          float2 n;
          dd::dot2(x.x, x.y, s1.x, s1.y, nb.x, nb.y, s2.x, s2.y, n.x, n.y);   // x mu1 - beta mu2
          s2 = s1;
          s1 = n;
          const float am = fmaxf(fabsf(s1.x), fabsf(s2.x));
          if (am > 0x1p32f) {
            s1.x *= 0x1p-64f; s1.y *= 0x1p-64f; s2.x *= 0x1p-64f; s2.y *= 0x1p-64f;
            et += 64;
          } else if (am < 0x1p-32f && am > 0.f) {
            s1.x *= 0x1p64f; s1.y *= 0x1p64f; s2.x *= 0x1p64f; s2.y *= 0x1p64f;
            et -= 64;
          }
        }
        if (valid) {
          const float2 c1 = s_pc[jj][0], c2 = s_pc[jj][1], c3 = s_pc[jj][2], c4 = s_pc[jj][3];
          float2 u, t, c4x, v, l1, l2;
          dd::mul(s2.x, s2.y, c1.x, c1.y, u.x, u.y);                          // mu2 c1
          dd::dot2(c2.x, c2.y, is2.x, is2.y, c3.x, c3.y, 1.f, 0.f, t.x, t.y);  // c2/sin^2 + c3
          dd::dot2(u.x, u.y, bw.x, bw.y, -s1.x, -s1.y, t.x, t.y, l1.x, l1.y);
          dd::mul(c4.x, c4.y, x.x, x.y, c4x.x, c4x.y);
          dd::dot2(u.x, u.y, 1.f, 0.f, -s1.x, -s1.y, c4x.x, c4x.y, v.x, v.y);
          dd::mul(v.x, v.y, cw.x, cw.y, l2.x, l2.y);                          // (..) m/sin^2
          uint16_t d[4];
          bad |= tc::digits4_df(l1.x, l1.y, s_erow[jj] - et, d);
          pk1 = (unsigned long long)d[0] | ((unsigned long long)d[1] << 16) |
                ((unsigned long long)d[2] << 32) | ((unsigned long long)d[3] << 48);
          bad |= tc::digits4_df(l2.x, l2.y, s_erow[jj] - et, d);
          pk2 = (unsigned long long)d[0] | ((unsigned long long)d[1] << 16) |
                ((unsigned long long)d[2] << 32) | ((unsigned long long)d[3] << 48);
        }
      }
      Sidx(0, jj & 1, jj >> 1, tid) = pk1;
      Sidx(1, jj & 1, jj >> 1, tid) = pk2;
    }
    __syncthreads();
    const int t = lb / (2 * kRows);
    const int rowt0 = (lb % (2 * kRows)) >> 1;
    for (int u = tid; u < 2 * 2 * (kPolBlock / 2) * (kSCRings / 8); u += 128) {
      const int r8 = u & 7, khalf = (u >> 3) & 1, rg = (u >> 4) & 1, ks = (u >> 5) & 7,
                par = (u >> 8) & 1, part = u >> 9;
      const int gks = rb * (kSCRings / kKStep) + ks;
      if (gks >= nks) continue;
      const int row = rg * 8 + r8;
      const unsigned long long* src = &Sidx(part, par, row, ks * kKStep + khalf * 8);
      unsigned long long v[8];
#pragma unroll
      for (int i = 0; i < 8; i += 2) {
        const ulonglong2 w = *reinterpret_cast<const ulonglong2*>(src + i);
        v[i] = w.x;
        v[i + 1] = w.y;
      }
      const int rowt = rowt0 + row;
      unsigned char* tile =
          base + (((size_t)(par * ntiles + t) * 2 + part) * nks + gks) * kSlices * kATileBytes +
          (rowt >> 3) * 256 + khalf * 128 + (rowt & 7) * 16;
#pragma unroll
      for (int d = 0; d < kSlices; ++d) {
        uint32_t h[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) h[i] = (uint32_t)(v[i] >> (16 * d)) & 0xFFFFu;
        uint4 o;
        o.x = h[0] | (h[1] << 16);
        o.y = h[2] | (h[3] << 16);
        o.z = h[4] | (h[5] << 16);
        o.w = h[6] | (h[7] << 16);
        *reinterpret_cast<uint4*>(tile + (size_t)d * kATileBytes) = o;
      }
    }
    stage(lb + kPolBlock);
    __syncthreads();
  }
  if (bad) atomicOr(a.err, tc::kErrRange);
}

// Persistent, like k_split_gemm: one CTA per SM walks work units (q, l-tile, parity, field
// E|B, 64-map group), the group fastest.  A unit runs, per part of <= 64 k-steps (1024 rings
// keep levels 0 and 1 exact), the lambda1 pass then the lambda2 pass through the same TMEM
// accumulators; the epilogue of each pass stores or adds (fire-and-forget reductions; the same
// thread handles every pass of an element, so the result is deterministic).
constexpr int kStagesP = 6;
constexpr uint32_t kStageBytesP = 2 * kSlices * kATileBytes;    // 32 KB: A then B
constexpr int kPartStepsP = kKChunk / kKStep;

struct GemmPArgs {
  int lmax, nnorth, ngroups, q0, ntmax, accumulate, which, nunits;
  int part_steps;        // k-steps per ring part, <= kPartStepsP (the plan's tile choice)
  size_t row_bytes;
  const int* ring_i0;
  const long long* lam_off;
  const FshtLamRow* tab;
  const unsigned char* lbuf;
  const unsigned char* WSQ;
  const unsigned char* WSU;
  const int* EBQ;
  const int* EBU;
  double* almE;
  double* almB;
  int ld, k0, kc;
  double pa;
  int* err;
};

struct __align__(8) GemmPSmemHdr {
  uint64_t full[kStagesP], empty[kStagesP], tfull, tempty, fin;
  uint32_t tmem;
  int abort;
};

// One work unit; nks = 0: nothing to do (l-tile beyond lmax - m, or a field not asked for).
struct GemmPUnit {
  int g, field, p, t, qi, m, nks, ntiles, lt0;
};

__device__ __forceinline__ GemmPUnit gemm_pol_unit(const GemmPArgs& a, int u) {
  GemmPUnit w;
  w.g = u % a.ngroups;
  int r = u / a.ngroups;
  w.field = r & 1;               // 0: E, 1: B
  r >>= 1;
  w.p = r & 1;
  r >>= 1;
  w.t = r % a.ntmax;
  w.qi = r / a.ntmax;
  w.m = m_of_q(a.q0 + w.qi, a.lmax);
  const int K = a.nnorth - a.ring_i0[w.m];
  w.ntiles = (a.lmax - w.m + 1 + 2 * kRows - 1) / (2 * kRows);
  w.nks = (w.t < w.ntiles && (a.which & (1 << w.field))) ? (K + kKStep - 1) / kKStep : 0;
  w.lt0 = w.m + w.t * 2 * kRows;
  return w;
}

__global__ void __launch_bounds__(kThreadsG, 1) k_split_gemm_pol(GemmPArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ GemmPSmemHdr h;
  __shared__ int s_ce[2][kCols];       // column exponents (e - 12) per pass of the unit

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  volatile int* abort = &h.abort;
  if (tid == 0) {
    for (int s = 0; s < kStagesP; ++s) {
      tc::mbar_init(&h.full[s], 1);
      tc::mbar_init(&h.empty[s], 1);
    }
    tc::mbar_init(&h.tfull, 1);
    tc::mbar_init(&h.tempty, kEpiThreads);
    tc::mbar_init(&h.fin, 1);
    h.abort = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(&h.tmem, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = h.tmem;

  uint32_t n_loaded = 0;
  if (tid == kEpiThreads) {
    // producer: per part, the lambda1 k-steps (B = the field's own map) then the lambda2
    // k-steps (B = the other map, opposite parity)
    uint32_t i = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < a.nunits && ok && !*abort; u += gridDim.x) {
      const GemmPUnit w = gemm_pol_unit(a, u);
      if (w.nks == 0) continue;
      const unsigned char* lam =
          a.lbuf + (size_t)(2 * (a.lam_off[a.q0 + w.qi] - a.lam_off[a.q0])) * kSlices * kATileBytes;
      const unsigned char* ws[2] = {w.field == 0 ? a.WSQ : a.WSU, w.field == 0 ? a.WSU : a.WSQ};
      const int bpar[2] = {w.p, 1 - w.p};
      for (int ks0 = 0; ks0 < w.nks && ok; ks0 += a.part_steps) {
        const int nk = min(w.nks - ks0, a.part_steps);
        for (int part = 0; part < 2 && ok; ++part) {
          for (int k = 0; k < nk; ++k, ++i) {
            const int ks = ks0 + k;
            const uint32_t st = i % kStagesP;
            if (!tc::mbar_wait(&h.empty[st], ((i / kStagesP) & 1) ^ 1, abort)) {
              ok = false;
              break;
            }
            unsigned char* dst = smem + st * kStageBytesP;
            const unsigned char* asrc =
                lam + (((size_t)(w.p * w.ntiles + w.t) * 2 + part) * w.nks + ks) * kSlices *
                          kATileBytes;
            const unsigned char* bsrc =
                ws[part] + (((size_t)w.qi * 2 + bpar[part]) * a.ngroups + w.g) * a.row_bytes +
                (size_t)ks * kSlices * kBTileBytes;
            tc::mbar_arrive_expect_tx(&h.full[st], kStageBytesP);
            tc::bulk_g2s(dst, asrc, kSlices * kATileBytes, &h.full[st]);
            tc::bulk_g2s(dst + kSlices * kATileBytes, bsrc, kSlices * kBTileBytes, &h.full[st]);
            ++n_loaded;
          }
        }
      }
    }
  } else if (tid == kEpiThreads + 32) {
    // UMMA issuer: one accumulation pass per (part of k-steps, lambda1 | lambda2)
    const uint32_t idesc = tc::umma_idesc_bf16(kRows, kCols);
    const uint32_t s_u = tc::smem_u32(smem);
    uint32_t i = 0, np = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < a.nunits && ok && !*abort; u += gridDim.x) {
      const GemmPUnit w = gemm_pol_unit(a, u);
      for (int ks0 = 0; ks0 < w.nks && ok; ks0 += a.part_steps) {
        const int nk = min(w.nks - ks0, a.part_steps);
        for (int part = 0; part < 2 && ok; ++part, ++np) {
          if (np > 0 && !tc::mbar_wait(&h.tempty, (np - 1) & 1, abort)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          for (int k = 0; k < nk; ++k, ++i) {
            const uint32_t st = i % kStagesP;
            if (!tc::mbar_wait(&h.full[st], (i / kStagesP) & 1, abort)) {
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint32_t abase = s_u + st * kStageBytesP;
            const uint32_t bbase = abase + kSlices * kATileBytes;
#pragma unroll
            for (int lev = 0; lev <= 3; ++lev) {
#pragma unroll
              for (int aa = 0; aa <= lev; ++aa) {
                const uint64_t ad = tc::umma_desc(abase + aa * kATileBytes, 128, 256);
                const uint64_t bd = tc::umma_desc(bbase + (lev - aa) * kBTileBytes, 128, 256);
                tc::umma_bf16(tmem + lev * kCols, ad, bd, idesc, (k > 0 || aa > 0) ? 1u : 0u);
              }
            }
            tc::umma_commit(&h.empty[st]);
          }
          if (ok) tc::umma_commit(&h.tfull);
        }
      }
    }
  } else if (tid < kEpiThreads) {
    // epilogue (warps 0-7), row = TMEM lane (warp % 4: lane quarter, warp / 4: half of the
    // columns).  No early exit: the epilogue threads must meet at every named barrier, so
    // after an expired wait (abort) the remaining passes are walked idle.
    const int lane = tid & 31;
    const int row0 = (warp & 3) << 5;              // this warp's 32 rows (its TMEM lane quarter)
    const int row = row0 + lane;
    // tgt: the alm component (Re 0, Im 1) this warp writes, in every pass.  The first pass
    // maps accumulator columns (Re, Im) to (Re, Im), the second (factor +-i) to (Im, Re), so in
    // the second pass the warp reads the other half of the columns: every element then has one
    // writer, whose store (first pass) and adds (later passes) are in its program order.
    const int tgt = warp >> 2;
    const long long L1 = a.lmax + 1;
    const uint32_t lane_base = tmem + ((uint32_t)row0 << 16);
    double* stg = reinterpret_cast<double*>(smem + (size_t)kStagesP * kStageBytesP) +
                  (size_t)warp * kStgWarpDoubles;
    uint32_t np = 0;
    for (int u = blockIdx.x; u < a.nunits; u += gridDim.x) {
      const GemmPUnit w = gemm_pol_unit(a, u);
      if (w.nks == 0) continue;
      {
        const int* eb[2] = {w.field == 0 ? a.EBQ : a.EBU, w.field == 0 ? a.EBU : a.EBQ};
        const int bpar[2] = {w.p, 1 - w.p};
        int e[2] = {0, 0};
        if (tid < kCols)
          for (int part = 0; part < 2; ++part)
            e[part] =
                eb[part][(((long long)w.qi * 2 + bpar[part]) * a.ngroups + w.g) * kCols + tid];
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
        if (tid < kCols)
          for (int part = 0; part < 2; ++part)
            s_ce[part][tid] = (e[part] == kEmptyExp) ? kEmptyExp : e[part] - 12;
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
      }
      const int l = w.lt0 + w.p + 2 * row;
      const bool rowok = l <= a.lmax;
      float rh = 0.f, rl = 0.f;
      int re = 0;
      if (rowok) {
        const FshtLamRow rw = a.tab[tri_off(w.m, a.lmax) + (l - w.m)];
        factor_pair(-rw.dm * a.pa, rh, rl);
        re = rw.erow + rw.dx;
      }
      double* alm = w.field == 0 ? a.almE : a.almB;
      for (int ks0 = 0; ks0 < w.nks; ks0 += a.part_steps) {
        for (int part = 0; part < 2; ++part) {
          bool ok = tc::mbar_wait(&h.tfull, np & 1, abort);
          ok = __all_sync(0xffffffffu, ok);
          ++np;
          if (!ok) continue;
          tc::tc_fence_after();
          const bool add = ks0 > 0 || part > 0 || a.accumulate;
          // part 0: (Re, Im) -> (Re, Im).  part 1 (factor +i for E, -i for B):
          //   E: Re <- -Im, Im <- +Re;   B: Re <- +Im, Im <- -Re
          const int comp = part == 0 ? tgt : 1 - tgt;     // the accumulator half read
          const bool neg = part == 1 && ((w.field == 0) == (comp == 1));
          const int cbeg = comp * (kCols / 2);
          const bool tgt_ok = !(tgt == 1 && w.m == 0);    // Im of m = 0 does not exist
          // drain first (as in k_split_gemm): the warp's 64 columns leave TMEM as FP32 (hi, lo)
          // pairs and TMEM goes back to the UMMA issuer before the FP64 work and the stores
          float hh[kCols / 2], ll[kCols / 2];
#pragma unroll
          for (int c = 0; c < kCols / 2; c += 8) {
            uint32_t v0[8], v1[8], v2[8], v3[8];
            tc::tmem_ld8(lane_base + 0 * kCols + cbeg + c, v0);
            tc::tmem_ld8(lane_base + 1 * kCols + cbeg + c, v1);
            tc::tmem_ld8(lane_base + 2 * kCols + cbeg + c, v2);
            tc::tmem_ld8(lane_base + 3 * kCols + cbeg + c, v3);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 8; ++j)
              combine_levels_pair(v0[j], v1[j], v2[j], v3[j], hh[c + j], ll[c + j]);
          }
          tc::tc_fence_before();
          tc::mbar_arrive(&h.tempty);
#pragma unroll
          for (int cr = 0; cr < kCols / 2; cr += 16) {
            const int c0 = cbeg + cr;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const double uu =
                  rowok ? pair_scaled(hh[cr + j], ll[cr + j], rh, rl, re + s_ce[part][c0 + j])
                        : 0.0;
              stg[stg_at(lane, j)] = neg ? -uu : uu;
            }
            __syncwarp();
            // the block back out by rows (lanes 0-15 one row, 16-31 the next), as fire-and-forget
            // stores / reductions
            const int cc = lane & 15;
            const int k = w.g * kGroupMaps + ((c0 + cc) & 63);
            if (tgt_ok && k < a.kc) {
#pragma unroll 4
              for (int i = 0; i < 16; ++i) {
                const int r = 2 * i + (lane >> 4);
                const int lr = w.lt0 + w.p + 2 * (row0 + r);
                if (lr <= a.lmax) {
                  const long long rowidx =
                      tgt == 0 ? ((long long)w.m * L1 + lr) : ((L1 - w.m) * L1 + (lr - w.m));
                  double* dst = alm + rowidx * a.ld + a.k0 + k;
                  const double v = stg[stg_at(r, cc)];
                  if (add) atomicAdd(dst, v);
                  else *dst = v;
                }
              }
            }
            __syncwarp();
          }
        }
      }
    }
  }
  if (tid == kEpiThreads + 32) {
    tc::umma_commit(&h.fin);
    for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
      if (tc::mbar_try_wait(&h.fin, 0)) break;
  }
  if (tid == kEpiThreads) {
    for (uint32_t d = 0; d < (uint32_t)kStagesP && d < n_loaded; ++d) {
      const uint32_t i = n_loaded - 1 - d;
      for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
        if (tc::mbar_try_wait(&h.full[i % kStagesP], (i / kStagesP) & 1)) break;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (tid == 0 && h.abort) atomicOr(a.err, tc::kErrTimeout);
}

// ------------------------------------------------------------------ spin-2 synthesis
// G_Q = -(lambda1 E + i lambda2 B), G_U = i lambda2 E - lambda1 B (sht_main.f90:1079-1147),
// north = even + odd l-m; south: lambda1 keeps the sign (-1)^(l-m), lambda2 takes the
// opposite one.  Ring-row tiles of lambda1 and lambda2 against one global scale (as in the
// spin-0 synthesis), the E and B alm tiles of k_slice_alm (with the 2^-8 planes, level 4
// folded in).

// grid (q in wave, 128-ring block), 128 threads = rings.  Tiles of m: (part, parity, ring
// block, l-step) x 4 digits at twice the spin-0 synthesis offset of q.
struct LamTPArgs {
  int lmax, nnorth, q0, eag;
  const double* cth;
  const double* sth;
  const double* pref;
  const int* ring_i0;
  const FshtLamRow* tab;
  const FshtPolRow* ptab;
  const long long* lam_offT;
  unsigned char* lbuf;
  int* err;
};

__global__ void __launch_bounds__(128) k_lambda_digits_T_pol(LamTPArgs a) {
  __shared__ float2 s_bd[32][2];          // -beta, Dm as df64 pairs
  __shared__ int s_dx[32];
  __shared__ float2 s_pc[32][4];          // c1..c4 as df64 pairs
  const int q = a.q0 + blockIdx.x;
  const int m = m_of_q(q, a.lmax);
  const int i0 = a.ring_i0[m];
  const int K = a.nnorth - i0;
  const int rb = blockIdx.y;
  if (rb * kSCRings >= K) return;
  const int tid = threadIdx.x;
  const int r = rb * kSCRings + tid;
  const bool valid = r < K;
  const int nrb = (K + kSCRings - 1) / kSCRings;
  const int nkl = ((a.lmax - m) / 2 + 1 + kKStep - 1) / kKStep;
  unsigned char* base =
      a.lbuf + (size_t)(2 * (a.lam_offT[q] - a.lam_offT[a.q0])) * kSlices * kATileBytes +
      (tid >> 3) * 256 + (tid & 7) * 16;
  const FshtLamRow* tab = a.tab + tri_off(m, a.lmax);
  const FshtPolRow* ptab = a.ptab + tri_off(m, a.lmax);
  auto pair = [](double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
  };
  // df64 recursion and lambda1 / lambda2 forms, as in k_lambda_digits_pol
  float2 x = make_float2(0.f, 0.f), is2 = x, bw = x, cw = x, s1 = x, s2 = x;
  int et = 0;
  if (valid) {
    int e, kx;
    const double sth = a.sth[i0 + r];
    const double xd = a.cth[i0 + r];
    const double inv_s2 = 1.0 / (sth * sth);
    double sd;
    rec_seed(sth, a.pref[m], m, sd, e);
    const double f = frexp(sd, &kx);
    et = 600 * e + kx;
    s1 = pair(f);
    x = pair(xd);
    is2 = pair(inv_s2);
    bw = pair(xd * inv_s2);
    cw = pair((double)m * inv_s2);
  }
  bool bad = false;
  for (int kl = 0; kl < nkl; ++kl) {
    __syncthreads();
    if (tid < 32 && m + kl * 32 + tid <= a.lmax) {
      const FshtLamRow rw = tab[kl * 32 + tid];
      const FshtPolRow c = ptab[kl * 32 + tid];
      s_bd[tid][0] = pair(-rw.beta);
      s_bd[tid][1] = pair(rw.dm);
      s_dx[tid] = rw.dx;
      s_pc[tid][0] = pair(c.c1);
      s_pc[tid][1] = pair(c.c2);
      s_pc[tid][2] = pair(c.c3);
      s_pc[tid][3] = pair(c.c4);
    }
    __syncthreads();
#pragma unroll 1
    for (int half = 0; half < 2; ++half) {
      uint32_t pk[2][2][kSlices][4];      // [part][parity][digit][word]
#pragma unroll
      for (int a0 = 0; a0 < 2; ++a0)
#pragma unroll
        for (int pp = 0; pp < 2; ++pp)
#pragma unroll
          for (int d = 0; d < kSlices; ++d)
#pragma unroll
            for (int w = 0; w < 4; ++w) pk[a0][pp][d][w] = 0;
#pragma unroll
      for (int jj = 0; jj < 16; ++jj) {
        const int j = kl * 32 + half * 16 + jj;
        uint16_t d1[4] = {0, 0, 0, 0}, d2[4] = {0, 0, 0, 0};
        if (m + j <= a.lmax) {
          const int jr = half * 16 + jj;
          if (j > 0) {
            const float2 nb = s_bd[jr][0];
            float2 n;
            dd::dot2(x.x, x.y, s1.x, s1.y, nb.x, nb.y, s2.x, s2.y, n.x, n.y);
            s2 = s1;
            s1 = n;
            const float am = fmaxf(fabsf(s1.x), fabsf(s2.x));
            if (am > 0x1p32f) {
              s1.x *= 0x1p-64f; s1.y *= 0x1p-64f; s2.x *= 0x1p-64f; s2.y *= 0x1p-64f;
              et += 64;
            } else if (am < 0x1p-32f && am > 0.f) {
              s1.x *= 0x1p64f; s1.y *= 0x1p64f; s2.x *= 0x1p64f; s2.y *= 0x1p64f;
              et -= 64;
            }
          }
          if (valid) {
            const float2 c1 = s_pc[jr][0], c2 = s_pc[jr][1], c3 = s_pc[jr][2], c4 = s_pc[jr][3];
            const float2 dm = s_bd[jr][1];
            float2 u, t, c4x, v, l1, l2;
            dd::mul(s2.x, s2.y, c1.x, c1.y, u.x, u.y);
            dd::dot2(c2.x, c2.y, is2.x, is2.y, c3.x, c3.y, 1.f, 0.f, t.x, t.y);
            dd::dot2(u.x, u.y, bw.x, bw.y, -s1.x, -s1.y, t.x, t.y, l1.x, l1.y);
            dd::mul(c4.x, c4.y, x.x, x.y, c4x.x, c4x.y);
            dd::dot2(u.x, u.y, 1.f, 0.f, -s1.x, -s1.y, c4x.x, c4x.y, v.x, v.y);
            dd::mul(v.x, v.y, cw.x, cw.y, l2.x, l2.y);
            dd::mul(l1.x, l1.y, dm.x, dm.y, l1.x, l1.y);
            dd::mul(l2.x, l2.y, dm.x, dm.y, l2.x, l2.y);
            bad |= tc::digits4_df(l1.x, l1.y, a.eag - et - s_dx[jr], d1);
            bad |= tc::digits4_df(l2.x, l2.y, a.eag - et - s_dx[jr], d2);
          }
        }
        const int par = jj & 1, slot = jj >> 1;
#pragma unroll
        for (int dd = 0; dd < kSlices; ++dd) {
          pk[0][par][dd][slot >> 1] |= (uint32_t)d1[dd] << (16 * (slot & 1));
          pk[1][par][dd][slot >> 1] |= (uint32_t)d2[dd] << (16 * (slot & 1));
        }
      }
#pragma unroll
      for (int part = 0; part < 2; ++part)
#pragma unroll
        for (int par = 0; par < 2; ++par)
#pragma unroll
          for (int dd = 0; dd < kSlices; ++dd) {
            uint4 o;
            o.x = pk[part][par][dd][0];
            o.y = pk[part][par][dd][1];
            o.z = pk[part][par][dd][2];
            o.w = pk[part][par][dd][3];
            *reinterpret_cast<uint4*>(
                base + ((((size_t)(part * 2 + par) * nrb + rb) * nkl + kl) * kSlices + dd) *
                           kATileBytes +
                half * 128) = o;
          }
    }
  }
  if (bad) atomicOr(a.err, tc::kErrRange);
}

// CTA = (group, ring block x l-chunk x field (Q, U), q): four passes through the same TMEM
// accumulators, each one (lambda part, alm field, parity) product added to G_N and G_S with
// its factor c in {-1, -i, +i} and south sign.
struct SynthPArgs {
  int lmax, nnorth, ngroups, q0, nrbmax, eag, nunits;
  size_t row_bytes;
  const int* ring_i0;
  const long long* lam_offT;
  const unsigned char* lbuf;
  const unsigned char* WSE;
  const unsigned char* WSB;
  const int* EBE;
  const int* EBB;
  double* WQ;      // double2 {G_N, G_S} as doubles
  double* WU;
  int kc;
  int* err;
};

constexpr int kStagesSP = 4;
constexpr uint32_t kStageBytesSP = kSlices * kATileBytes + kSynthBBytes;   // 44 KB
constexpr int kPartStepsSP = kKChunk / kKStep;

struct __align__(8) SynthPSmemHdr {
  uint64_t full[kStagesSP], empty[kStagesSP], tfull, tempty, fin;
  uint32_t tmem;
  int abort;
};

// One work unit (q, 128-ring block, field Q|U, 64-map group), the group fastest; nkl = 0:
// nothing to do.
struct SynthPUnit {
  int g, f, rb, qi, m, i0, K, nrb, nkl;
};

__device__ __forceinline__ SynthPUnit synth_pol_unit(const SynthPArgs& a, int u) {
  SynthPUnit w;
  w.g = u % a.ngroups;
  int r = u / a.ngroups;
  w.f = r & 1;
  r >>= 1;
  w.rb = r % a.nrbmax;
  w.qi = r / a.nrbmax;
  w.m = m_of_q(a.q0 + w.qi, a.lmax);
  w.i0 = a.ring_i0[w.m];
  w.K = a.nnorth - w.i0;
  w.nrb = (w.K + kSCRings - 1) / kSCRings;
  w.nkl = w.rb < w.nrb ? ((a.lmax - w.m) / 2 + 1 + kKStep - 1) / kKStep : 0;
  return w;
}

// pass t of field f: lambda part, alm field (0 E, 1 B), parity, factor c (0: -1, 1: -i,
// 2: +i) and south sign
__device__ __forceinline__ void synth_pol_pass(int f, int t, int& part, int& fld, int& par,
                                               int& c, int& sgn_s) {
  par = t & 1;
  const int second = t >> 1;
  if (f == 0) {          // G_Q = -(l1 E) - i (l2 B)
    part = second;       // l1 then l2
    fld = second;        // E then B
    c = second ? 1 : 0;
  } else {               // G_U = i (l2 E) - (l1 B)
    part = 1 - second;   // l2 then l1
    fld = second;        // E then B
    c = second ? 0 : 2;
  }
  const int s1 = par ? -1 : 1;              // lambda1: (-1)^(l-m)
  sgn_s = (part == 0) ? s1 : -s1;           // lambda2: the opposite sign
}

// Persistent like the analysis contractions: one CTA per SM walks the units; per part of
// <= 64 l-steps the four passes (lambda part x alm field x parity, synth_pol_pass) run through
// the same TMEM accumulators.  The first pass of a unit writes both components of G_N and G_S,
// every later pass adds as fire-and-forget reductions from the thread that owns the element
// (deterministic, no clearing of W).  Warps 0-7: epilogue, warp 8 lane 0: copies, warp 9
// lane 0: UMMAs.
__global__ void __launch_bounds__(kThreadsG, 1) k_split_synth_pol(SynthPArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ SynthPSmemHdr h;
  __shared__ int s_ce[4][kCols];       // column exponents EAG + e - 12 per pass

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  volatile int* abort = &h.abort;
  if (tid == 0) {
    for (int s = 0; s < kStagesSP; ++s) {
      tc::mbar_init(&h.full[s], 1);
      tc::mbar_init(&h.empty[s], 1);
    }
    tc::mbar_init(&h.tfull, 1);
    tc::mbar_init(&h.tempty, kEpiThreads);
    tc::mbar_init(&h.fin, 1);
    h.abort = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(&h.tmem, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = h.tmem;

  uint32_t n_loaded = 0;
  if (tid == kEpiThreads) {
    uint32_t i = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < a.nunits && ok && !*abort; u += gridDim.x) {
      const SynthPUnit w = synth_pol_unit(a, u);
      if (w.nkl == 0) continue;
      const unsigned char* lam =
          a.lbuf + (size_t)(2 * (a.lam_offT[a.q0 + w.qi] - a.lam_offT[a.q0])) * kSlices * kATileBytes;
      for (int kl0 = 0; kl0 < w.nkl && ok; kl0 += kPartStepsSP) {
        const int nk = min(w.nkl - kl0, kPartStepsSP);
        for (int t = 0; t < 4 && ok; ++t) {
          int part, fld, par, c, sg;
          synth_pol_pass(w.f, t, part, fld, par, c, sg);
          for (int kk = kl0; kk < kl0 + nk; ++kk, ++i) {
            const uint32_t st = i % kStagesSP;
            if (!tc::mbar_wait(&h.empty[st], ((i / kStagesSP) & 1) ^ 1, abort)) {
              ok = false;
              break;
            }
            unsigned char* dst = smem + st * kStageBytesSP;
            const unsigned char* asrc =
                lam + ((((size_t)(part * 2 + par) * w.nrb + w.rb) * w.nkl + kk) * kSlices) *
                          kATileBytes;
            const unsigned char* bsrc =
                (fld ? a.WSB : a.WSE) +
                (((size_t)w.qi * 2 + par) * a.ngroups + w.g) * a.row_bytes +
                (size_t)kk * kSynthBBytes;
            tc::mbar_arrive_expect_tx(&h.full[st], kStageBytesSP);
            tc::bulk_g2s(dst, asrc, kSlices * kATileBytes, &h.full[st]);
            tc::bulk_g2s(dst + kSlices * kATileBytes, bsrc, kSynthBBytes, &h.full[st]);
            ++n_loaded;
          }
        }
      }
    }
  } else if (tid == kEpiThreads + 32) {
    const uint32_t idesc = tc::umma_idesc_bf16(kRows, kCols);
    const uint32_t s_u = tc::smem_u32(smem);
    uint32_t i = 0, np = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < a.nunits && ok && !*abort; u += gridDim.x) {
      const SynthPUnit w = synth_pol_unit(a, u);
      for (int kl0 = 0; kl0 < w.nkl && ok; kl0 += kPartStepsSP) {
        const int nk = min(w.nkl - kl0, kPartStepsSP);
        for (int t = 0; t < 4 && ok; ++t, ++np) {
          if (np > 0 && !tc::mbar_wait(&h.tempty, (np - 1) & 1, abort)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          for (int k = 0; k < nk; ++k, ++i) {
            const uint32_t st = i % kStagesSP;
            if (!tc::mbar_wait(&h.full[st], (i / kStagesSP) & 1, abort)) {
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint32_t abase = s_u + st * kStageBytesSP;
            const uint32_t bbase = abase + kSlices * kATileBytes;
#pragma unroll
            for (int lev = 0; lev <= 3; ++lev) {
#pragma unroll
              for (int aa = 0; aa <= lev; ++aa) {
                const uint64_t ad = tc::umma_desc(abase + aa * kATileBytes, 128, 256);
                const uint64_t bd = tc::umma_desc(bbase + (lev - aa) * kBTileBytes, 128, 256);
                tc::umma_bf16(tmem + lev * kCols, ad, bd, idesc, (k > 0 || aa > 0) ? 1u : 0u);
              }
            }
#pragma unroll
            for (int aa = 1; aa <= 3; ++aa) {
              const uint64_t ad = tc::umma_desc(abase + aa * kATileBytes, 128, 256);
              const uint64_t bd =
                  tc::umma_desc(bbase + (kSlices - 1 + (4 - aa)) * kBTileBytes, 128, 256);
              tc::umma_bf16(tmem + 3 * kCols, ad, bd, idesc, 1u);
            }
            tc::umma_commit(&h.empty[st]);
          }
          if (ok) tc::umma_commit(&h.tfull);
        }
      }
    }
  } else if (tid < kEpiThreads) {
    // No early exit: the epilogue threads must meet at every named barrier.
    const int row = ((warp & 3) << 5) + (tid & 31);
    const int cbeg = (warp >> 2) * (kCols / 2);
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) << 5) << 16);
    uint32_t np = 0;
    for (int u = blockIdx.x; u < a.nunits; u += gridDim.x) {
      const SynthPUnit w = synth_pol_unit(a, u);
      if (w.nkl == 0) continue;
      {
        int e[4] = {0, 0, 0, 0};
        if (tid < kCols)
          for (int t = 0; t < 4; ++t) {
            int part, fld, par, c, sg;
            synth_pol_pass(w.f, t, part, fld, par, c, sg);
            const int* eb = fld ? a.EBB : a.EBE;
            e[t] = eb[(((long long)w.qi * 2 + par) * a.ngroups + w.g) * kCols + tid];
          }
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
        if (tid < kCols)
          for (int t = 0; t < 4; ++t)
            s_ce[t][tid] = (e[t] == kEmptyExp) ? kEmptyExp : a.eag + e[t] - 12;
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
      }
      const int rr = w.rb * kSCRings + row;
      const bool rowok = rr < w.K;
      const int i = w.i0 + rr;
      double* Wf = w.f ? a.WU : a.WQ;
      for (int kl0 = 0; kl0 < w.nkl; kl0 += kPartStepsSP) {
        for (int t = 0; t < 4; ++t) {
          int part, fld, par, c, sg;
          synth_pol_pass(w.f, t, part, fld, par, c, sg);
          bool ok = tc::mbar_wait(&h.tfull, np & 1, abort);
          ok = __all_sync(0xffffffffu, ok);
          ++np;
          if (!ok) continue;
          tc::tc_fence_after();
          const bool first = kl0 == 0 && t == 0;   // pass 0 writes both components
          for (int c0 = cbeg; c0 < cbeg + kCols / 2; c0 += 16) {
            uint32_t v0[16], v1[16], v2[16], v3[16];
            tc::tmem_ld16(lane_base + 0 * kCols + c0, v0);
            tc::tmem_ld16(lane_base + 1 * kCols + c0, v1);
            tc::tmem_ld16(lane_base + 2 * kCols + c0, v2);
            tc::tmem_ld16(lane_base + 3 * kCols + c0, v3);
            tc::tmem_wait_ld();
            if (c0 == cbeg + kCols / 2 - 16) {
              tc::tc_fence_before();
              tc::mbar_arrive(&h.tempty);
            }
            const int comp = c0 >> 6;
            // c D: -1: (-D.x, -D.y);  -i: (D.y, -D.x);  +i: (-D.y, D.x)
            int tgt = comp;
            bool neg = true;
            if (c == 1) {
              tgt = 1 - comp;
              neg = comp == 0;
            } else if (c == 2) {
              tgt = 1 - comp;
              neg = comp == 1;
            }
            if (!rowok) continue;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int cc = c0 + j;
              const int k = w.g * kGroupMaps + (cc & 63);
              if (k < a.kc) {
                const double uu =
                    levels_scaled(v0[j], v1[j], v2[j], v3[j], 1.f, 0.f, s_ce[t][cc]);
                const double v = neg ? -uu : uu;
                double* gn = Wf + ((((long long)w.m * a.nnorth + i) * a.kc + k) * 2) * 2 + tgt;
                double* gs = gn + 2;
                const double vs = sg < 0 ? -v : v;
                if (first) {
                  *gn = v;
                  *gs = vs;
                } else {
                  atomicAdd(gn, v);
                  atomicAdd(gs, vs);
                }
              }
            }
          }
        }
      }
    }
  }
  if (tid == kEpiThreads + 32) {
    tc::umma_commit(&h.fin);
    for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
      if (tc::mbar_try_wait(&h.fin, 0)) break;
  }
  if (tid == kEpiThreads) {
    for (uint32_t d = 0; d < (uint32_t)kStagesSP && d < n_loaded; ++d) {
      const uint32_t i = n_loaded - 1 - d;
      for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
        if (tc::mbar_try_wait(&h.full[i % kStagesSP], (i / kStagesSP) & 1)) break;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (tid == 0 && h.abort) atomicOr(a.err, tc::kErrTimeout);
}

}  // namespace

int fsht_split_pol_tables_init(fsht_plan* p) {
  const int lmax = p->lmax;
  const size_t ntab = (size_t)tri_off(lmax + 1, lmax);
  FSHT_CUDA_TRY(cudaMalloc(&p->d_poltab, sizeof(FshtPolRow) * (ntab ? ntab : 1)));
  k_pol_table<<<(lmax + 1 + 127) / 128, 128, 0, p->stream>>>(lmax, p->d_poltab);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

int fsht_launch_split_lambda_pol(fsht_plan* p, int w, unsigned char* lbuf, cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  if (wv[4] == 0) return FSHT_OK;
  LamPArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.q0 = wv[0];
  a.cth = p->d_cth;
  a.sth = p->d_sth;
  a.pref = p->d_pref;
  a.ring_i0 = p->d_ring_i0;
  a.tab = p->d_lamtab;
  a.ptab = p->d_poltab;
  a.lam_off = p->d_lam_off;
  a.lbuf = lbuf;
  a.err = p->d_err;
  FSHT_TRY(fsht_smem_limit((const void*)k_lambda_digits_pol, (size_t)(kPolStageBytes)));
  k_lambda_digits_pol<<<dim3(wv[1] - wv[0], wv[4]), 128, kPolStageBytes, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

int fsht_launch_split_gemm_pol(fsht_plan* p, int w, const unsigned char* WSQ, const int* EBQ,
                               const unsigned char* WSU, const int* EBU,
                               const unsigned char* lbuf, double* almE, double* almB,
                               int nmaps_total, int k0, int kc, int accumulate, int which,
                               cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  if (wv[3] == 0) return FSHT_OK;
  GemmPArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  a.q0 = wv[0];
  a.ntmax = wv[2];
  a.accumulate = accumulate;
  a.which = which;
  a.nunits = a.ngroups * 4 * a.ntmax * (wv[1] - wv[0]);
  a.row_bytes = ws_row_bytes(p->lmax, p->nnorth);
  a.ring_i0 = p->d_ring_i0;
  a.lam_off = p->d_lam_off;
  a.tab = p->d_lamtab;
  a.lbuf = lbuf;
  a.WSQ = WSQ;
  a.WSU = WSU;
  a.EBQ = EBQ;
  a.EBU = EBU;
  a.almE = almE;
  a.almB = almB;
  a.ld = nmaps_total;
  a.k0 = k0;
  a.kc = kc;
  a.pa = p->pa;
  a.err = p->d_err;
  a.part_steps =
      (p->split_part > 0 && p->split_part < kPartStepsP) ? p->split_part : kPartStepsP;
  const size_t sm = (size_t)kStagesP * kStageBytesP + kStgBytes;
  FSHT_TRY(fsht_smem_limit((const void*)k_split_gemm_pol, (size_t)(sm)));
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = a.nunits < nsm ? a.nunits : nsm;
  if (grid > 0) k_split_gemm_pol<<<grid, kThreadsG, sm, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

int fsht_launch_split_lambdaT_pol(fsht_plan* p, int w, unsigned char* lbuf, cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  if (wv[4] == 0) return FSHT_OK;
  LamTPArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.q0 = wv[0];
  a.eag = std::ilogb(std::sqrt((2.0 * p->lmax + 1.0) / (4.0 * M_PI)) * (1.0 + 0x1p-30)) + 1;
  a.cth = p->d_cth;
  a.sth = p->d_sth;
  a.pref = p->d_pref;
  a.ring_i0 = p->d_ring_i0;
  a.tab = p->d_lamtab;
  a.ptab = p->d_poltab;
  a.lam_offT = p->d_lam_offT;
  a.lbuf = lbuf;
  a.err = p->d_err;
  k_lambda_digits_T_pol<<<dim3(wv[1] - wv[0], wv[4]), 128, 0, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

int fsht_launch_split_synth_pol(fsht_plan* p, int w, const unsigned char* WSE, const int* EBE,
                                const unsigned char* WSB, const int* EBB,
                                const unsigned char* lbuf, double2* WQ, double2* WU, int kc,
                                cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  if (wv[4] == 0 || wv[6] == 0) return FSHT_OK;
  SynthPArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  a.q0 = wv[0];
  a.nrbmax = wv[4];
  a.nunits = a.ngroups * 2 * a.nrbmax * (wv[1] - wv[0]);
  a.eag = std::ilogb(std::sqrt((2.0 * p->lmax + 1.0) / (4.0 * M_PI)) * (1.0 + 0x1p-30)) + 1;
  a.row_bytes = ws_row_bytes(p->lmax, p->nnorth);
  a.ring_i0 = p->d_ring_i0;
  a.lam_offT = p->d_lam_offT;
  a.lbuf = lbuf;
  a.WSE = WSE;
  a.WSB = WSB;
  a.EBE = EBE;
  a.EBB = EBB;
  a.WQ = reinterpret_cast<double*>(WQ);
  a.WU = reinterpret_cast<double*>(WU);
  a.kc = kc;
  a.err = p->d_err;
  const size_t sm = (size_t)kStagesSP * kStageBytesSP;
  FSHT_TRY(fsht_smem_limit((const void*)k_split_synth_pol, (size_t)(sm)));
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = a.nunits < nsm ? a.nunits : nsm;
  if (grid > 0) k_split_synth_pol<<<grid, kThreadsG, sm, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}
