// Split-precision Legendre analysis on the 5th-generation tensor cores (tcgen05).
//
// The precision form of the reference's per-m analysis contraction (get_plm_recursive
// + mat2alm, src/get_plm_recursive.f90:17-98, src/sht_core.f90:30-89):
//   a_lm = pa sum_i lambda_lm(theta_i) P_m(i),  P = S (l-m even) or D (l-m odd).
// Both operands are written as four balanced base-256 digits against power-of-two
// scales (rows of lambda: 2^EA(l) with |lambda_lm| <= sqrt((2l+1)/4pi) < 2^EA(l);
// columns of P: 2^EB from the column maximum).  Digits are integers (|d0| <= 64,
// |d1..3| <= 128) that BF16 holds exactly, so every UMMA product is an exact integer.
// The ten digit products of level a+b <= 3 run as BF16 UMMAs with FP32 accumulation,
// one TMEM accumulator per level:
//   level 0 and level 1 sums stay below 2^24 over <= 1024 rings, so they are exact
//   (rings beyond 1024 go to another CTA: K-chunks, combined with FP64 atomics);
//   levels 2 and 3 carry weights 2^-16 and 2^-24, so FP32 rounding there is far
//   below the ~2^-31 representation error.
// The epilogue combines the four levels and applies the scales in FP64.  The
// recursion stays FP64 (exponent-rescaled, as in the plain path) and is computed on
// the fly: no P_lm table is materialised.  Max relative alm error against FP64:
// ~2e-8 (tests/test_gpu_split.py).
//
// CTA = (m-pair, parity, K-chunk of <= 1024 rings, 64-map group); it walks l in tiles
// of 128 rows of one parity (256 consecutive l) and keeps each ring's recursion state
// in shared memory between tiles.  Roles (192 threads): warps 0-3 run the recursion
// for 128 rings at a time and write lambda digits to shared memory, then read TMEM in
// the epilogue; warp 4 streams the pre-sliced P tiles with bulk async copies (TMA
// engine); warp 5 issues the UMMAs.
#include "common.cuh"
#include "tcgen05.cuh"

#include <cmath>

namespace {

constexpr int kRows = 128;          // UMMA M: rows of one parity per l-tile
constexpr int kCols = 128;          // UMMA N: 64 maps x {Re, Im}
constexpr int kGroupMaps = 64;
constexpr int kKStep = 16;          // rings per UMMA
constexpr int kSCRings = 128;       // rings per recursion super-chunk
constexpr int kSCSteps = kSCRings / kKStep;
constexpr int kKChunk = 1024;       // rings per CTA (keeps levels 0 and 1 exact)
constexpr int kSlices = 4;
constexpr int kStages = 3;
constexpr uint32_t kATileBytes = kRows * kKStep * 2;    // 4 KB per (k-step, digit)
constexpr uint32_t kBTileBytes = kCols * kKStep * 2;    // 4 KB per (k-step, digit)
constexpr uint32_t kABufBytes = kSCSteps * kSlices * kATileBytes;   // 128 KB
constexpr uint32_t kBStageBytes = kSlices * kBTileBytes;            // 16 KB
constexpr int kThreads = 192;
constexpr int kEmptyExp = -4000;    // column exponent of an all-zero column

struct RecConst {
  double a, b;
};

__device__ __forceinline__ RecConst rec_coeffs(int l, int m) {
  RecConst c;
  if (l == m) {          // state convention: lambda_m = -b prev = the seed
    c.a = 0.0;
    c.b = -1.0;
    return c;
  }
  const long long L = l, M = m;
  c.a = sqrt((double)((2 * L - 1) * (2 * L + 1)) / (double)(L * L - M * M));
  c.b = sqrt((double)((L - 1) * (L - 1) - M * M) / (double)((2 * L - 3) * (2 * L - 1))) * c.a;
  return c;
}

// Row scale: |lambda_lm(theta)| <= sqrt((2l+1)/(4 pi)) < 2^EA (the |Y_lm| bound).
__device__ __forceinline__ int row_exp(int l) {
  const double b = sqrt((2.0 * l + 1.0) / (4.0 * M_PI)) * (1.0 + 0x1p-30);
  return ilogb(b) + 1;
}

__device__ __forceinline__ void rec_seed(double sth, double pref, int m, double& v, int& e) {
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
  v = ldexp(rm, (int)(re - 600LL * e));
}

// ------------------------------------------------------------------ P digits
// grid (m, parity, group), 128 threads = columns (map = c & 63, Re/Im = c >> 6).
// WS tile (m, p, g, t, digit): 128 columns x 16 rings, core matrices (8 cols x 8
// rings, 128 B) at (c/8)*256 + (k/8)*128.  Rings beyond the kept range are zero.
struct SliceArgs {
  const double2* W;
  int kc, nnorth, ngroups, nks_max;
  const int* ring_i0;
  unsigned char* WS;
  int* EB;
};

__global__ void __launch_bounds__(128) k_slice_phase(SliceArgs a) {
  const int m = blockIdx.x, p = blockIdx.y, g = blockIdx.z;
  const int c = threadIdx.x;
  const int k = g * kGroupMaps + (c & 63);
  const int comp = c >> 6;
  const int i0 = a.ring_i0[m];
  const int K = a.nnorth - i0;
  const bool valid = k < a.kc;
  auto val = [&](int r) -> double {
    if (!valid || r >= K) return 0.0;
    const double2 w = a.W[(((long long)m * a.nnorth + i0 + r) * a.kc + k) * 2 + p];
    return comp ? w.y : w.x;
  };
  double mx = 0.0;
  for (int r = 0; r < K; ++r) mx = fmax(mx, fabs(val(r)));
  const int E = (mx > 0.0) ? ilogb(mx) + 1 : kEmptyExp;
  a.EB[(((long long)m * 2 + p) * a.ngroups + g) * kCols + c] = E;
  const int nks = (K + kKStep - 1) / kKStep;
  unsigned char* base =
      a.WS + (((size_t)(m * 2 + p) * a.ngroups + g) * a.nks_max) * kSlices * kBTileBytes;
  for (int t = 0; t < nks; ++t) {
    for (int half = 0; half < 2; ++half) {
      uint16_t s[kSlices][8];
      for (int j = 0; j < 8; ++j) {
        uint16_t q[4] = {0, 0, 0, 0};
        if (E != kEmptyExp) tc::digits4(val(t * kKStep + half * 8 + j), E, q);
        for (int sl = 0; sl < kSlices; ++sl) s[sl][j] = q[sl];
      }
      for (int sl = 0; sl < kSlices; ++sl) {
        uint4 pk;
        pk.x = s[sl][0] | ((uint32_t)s[sl][1] << 16);
        pk.y = s[sl][2] | ((uint32_t)s[sl][3] << 16);
        pk.z = s[sl][4] | ((uint32_t)s[sl][5] << 16);
        pk.w = s[sl][6] | ((uint32_t)s[sl][7] << 16);
        unsigned char* tile = base + ((size_t)t * kSlices + sl) * kBTileBytes;
        *reinterpret_cast<uint4*>(tile + (c >> 3) * 256 + half * 128 + (c & 7) * 16) = pk;
      }
    }
  }
}

// ------------------------------------------------------------------ analysis
struct SplitArgs {
  int lmax, nnorth, ngroups, nks_max, nkc;
  const double* cth;
  const double* sth;
  const double* pref;
  const int* ring_i0;
  const unsigned char* WS;
  const int* EB;
  double* alm;
  int ld, k0, kc;      // alm map extent, chunk offset, maps in the chunk
  double pa;
  int accumulate;      // add into alm (iterations); with nkc > 1 alm is pre-zeroed
  int* err;
};

struct __align__(8) SplitSmemHdr {
  uint64_t bfull[kStages], bempty[kStages], afull, aempty, tfull, tempty, fin;
  uint32_t tmem;
  int abort;
};

__global__ void __launch_bounds__(kThreads, 1) k_analysis_split(SplitArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;                                     // 128 KB
  unsigned char* sB = smem + kABufBytes;                        // 3 x 16 KB
  double* st_cur = reinterpret_cast<double*>(sB + kStages * kBStageBytes);
  double* st_prev = st_cur + kKChunk;
  int* st_e = reinterpret_cast<int*>(st_prev + kKChunk);
  __shared__ SplitSmemHdr h;
  __shared__ RecConst s_rc[2 * kRows];
  __shared__ int s_ea[kRows];
  __shared__ double s_cs[kCols];

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int p = blockIdx.y / a.nkc;
  const int kci = blockIdx.y % a.nkc;
  const int g = blockIdx.z;
  volatile int* abort = &h.abort;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&h.bfull[s], 1);
      tc::mbar_init(&h.bempty[s], 1);
    }
    tc::mbar_init(&h.afull, kSCRings);
    tc::mbar_init(&h.aempty, 1);
    tc::mbar_init(&h.tfull, 1);
    tc::mbar_init(&h.tempty, 128);
    tc::mbar_init(&h.fin, 1);
    h.abort = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(&h.tmem, 512);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = h.tmem;
  const uint32_t idesc = tc::umma_idesc_bf16(kRows, kCols);

  // per-thread counters carrying mbarrier phases across m passes and l-tiles
  uint32_t q_load = 0, q_mma = 0, sc_cnt = 0, tile_cnt = 0;

  for (int pass = 0; pass < 2; ++pass) {
    const int m = pass == 0 ? (int)blockIdx.x : a.lmax - (int)blockIdx.x;
    if (pass == 1 && m == (int)blockIdx.x) break;
    const int i0 = a.ring_i0[m];
    const int Ktot = a.nnorth - i0;
    const int r0 = kci * kKChunk;                 // first ring (relative to i0) of this chunk
    const int K = min(kKChunk, Ktot - r0);        // rings in this chunk
    if (K <= 0) continue;
    const int t0 = r0 / kKStep;                   // first global k-step
    const int nks = (K + kKStep - 1) / kKStep;
    const int nsc = (K + kSCRings - 1) / kSCRings;
    const int ntiles = (a.lmax - m + 1 + 2 * kRows - 1) / (2 * kRows);
    const unsigned char* wsb =
        a.WS + (((size_t)(m * 2 + p) * a.ngroups + g) * a.nks_max) * kSlices * kBTileBytes;
    if (tid < 128) {
      for (int r = tid; r < K; r += 128) {
        double v;
        int e;
        rec_seed(a.sth[i0 + r0 + r], a.pref[m], m, v, e);
        st_cur[r] = 0.0;   // lambda_{m-1}
        st_prev[r] = v;    // the seed, consumed by the l = m step (a = 0, b = -1)
        st_e[r] = e;
      }
      {
        const int c = tid;
        const int eb = a.EB[(((long long)m * 2 + p) * a.ngroups + g) * kCols + c];
        s_cs[c] = (eb == kEmptyExp) ? 0.0 : ldexp(a.pa, eb - 12);
      }
    }
    __syncthreads();

    for (int tt = 0; tt < ntiles; ++tt) {
      const int lt0 = m + tt * 2 * kRows;
      if (tid < 128) {
        for (int j = tid; j < 2 * kRows; j += 128) {
          const int l = lt0 + j;
          s_rc[j] = (l <= a.lmax) ? rec_coeffs(l, m) : RecConst{0.0, 0.0};
        }
        s_ea[tid] = row_exp(lt0 + p + 2 * tid);
        asm volatile("bar.sync 1, 128;" ::: "memory");
        // ---------------- producers: lambda digits for 128 rings at a time
        for (int sc = 0; sc < nsc; ++sc, ++sc_cnt) {
          if (!tc::mbar_wait(&h.aempty, (sc_cnt & 1) ^ 1, abort)) break;
          const int r = sc * kSCRings + tid;
          const int ks = tid / kKStep, kk = tid % kKStep;
          unsigned char* col = sA + ks * kSlices * kATileBytes + (kk >> 3) * 128 + (kk & 7) * 2;
          if (r < K) {
            double cur = st_cur[r], prev = st_prev[r];
            int e = st_e[r];
            const double cth = a.cth[i0 + r0 + r];
            for (int j2 = 0; j2 < 2 * kRows; ++j2) {
              const int l = lt0 + j2;
              double lam = 0.0;
              if (l <= a.lmax) {
                const double nx = s_rc[j2].a * cth * cur - s_rc[j2].b * prev;
                prev = cur;
                cur = nx;
                if (e < 0 && fabs(cur) > 0x1p300) {
                  cur *= 0x1p-600;
                  prev *= 0x1p-600;
                  ++e;
                }
                lam = (e == 0) ? cur : 0.0;
              }
              if ((j2 & 1) == p) {
                const int row = j2 >> 1;
                uint16_t dg[4];
                tc::digits4(lam, s_ea[row], dg);
                unsigned char* dst = col + (row >> 3) * 256 + (row & 7) * 16;
#pragma unroll
                for (int s = 0; s < kSlices; ++s)
                  *reinterpret_cast<uint16_t*>(dst + s * kATileBytes) = dg[s];
              }
            }
            st_cur[r] = cur;
            st_prev[r] = prev;
            st_e[r] = e;
          } else {
            for (int row = 0; row < kRows; ++row) {
              unsigned char* dst = col + (row >> 3) * 256 + (row & 7) * 16;
#pragma unroll
              for (int s = 0; s < kSlices; ++s)
                *reinterpret_cast<uint16_t*>(dst + s * kATileBytes) = 0;
            }
          }
          tc::fence_proxy_async();
          tc::mbar_arrive(&h.afull);
        }
      } else if (tid == 128) {
        // ---------------- P tiles: bulk async copies, kStages-deep ring
        for (int t = 0; t < nks; ++t, ++q_load) {
          const uint32_t st = q_load % kStages;
          if (!tc::mbar_wait(&h.bempty[st], ((q_load / kStages) & 1) ^ 1, abort)) break;
          tc::mbar_arrive_expect_tx(&h.bfull[st], kBStageBytes);
          tc::bulk_g2s(sB + st * kBStageBytes, wsb + (size_t)(t0 + t) * kSlices * kBTileBytes,
                       kBStageBytes, &h.bfull[st]);
        }
      } else if (tid == 160) {
        // ---------------- UMMA issue: level L digit products into accumulator L
        bool ok = tc::mbar_wait(&h.tempty, (tile_cnt & 1) ^ 1, abort);
        tc::tc_fence_after();
        const uint32_t sA_u = tc::smem_u32(sA), sB_u = tc::smem_u32(sB);
        int t = 0;
        uint32_t started = 0;   // bit L: accumulator L written in this tile
        for (int sc = 0; ok && sc < nsc; ++sc) {
          ok = tc::mbar_wait(&h.afull, (sc_cnt + sc) & 1, abort);
          if (!ok) break;
          tc::tc_fence_after();
          for (int ks = 0; ks < kSCSteps && t < nks; ++ks, ++t, ++q_mma) {
            const uint32_t st = q_mma % kStages;
            ok = tc::mbar_wait(&h.bfull[st], (q_mma / kStages) & 1, abort);
            if (!ok) break;
            tc::tc_fence_after();
            const uint32_t abase = sA_u + ks * kSlices * kATileBytes;
            const uint32_t bbase = sB_u + st * kBStageBytes;
#pragma unroll
            for (int lev = 0; lev <= 3; ++lev) {
#pragma unroll
              for (int aa = 0; aa <= lev; ++aa) {
                const int bb = lev - aa;
                const uint64_t ad = tc::umma_desc(abase + aa * kATileBytes, 128, 256);
                const uint64_t bd = tc::umma_desc(bbase + bb * kBTileBytes, 128, 256);
                tc::umma_bf16(tmem + lev * kCols, ad, bd, idesc, (started >> lev) & 1u);
                started |= 1u << lev;
              }
            }
            tc::umma_commit(&h.bempty[st]);
          }
          tc::umma_commit(&h.aempty);
        }
        tc::umma_commit(&h.tfull);
      }
      if (tid >= 128) sc_cnt += nsc;   // the producers advanced it in their loop
      // ---------------- epilogue (warps 0-3): TMEM -> alm
      if (tid < 128) {
        bool ok = tc::mbar_wait(&h.tfull, tile_cnt & 1, abort);
        ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-collective
        tc::tc_fence_after();
        const int row = (warp << 5) + (tid & 31);
        const int l = lt0 + p + 2 * row;
        const bool rowok = l <= a.lmax;
        if (ok) {
          const double rs = ldexp(1.0, s_ea[row]);
          const long long L1 = a.lmax + 1;
          const uint32_t lane_base = tmem + ((uint32_t)(warp << 5) << 16);
          for (int c0 = 0; c0 < kCols; c0 += 16) {
            uint32_t v0[16], v1[16], v2[16], v3[16];
            tc::tmem_ld16(lane_base + 0 * kCols + c0, v0);
            tc::tmem_ld16(lane_base + 1 * kCols + c0, v1);
            tc::tmem_ld16(lane_base + 2 * kCols + c0, v2);
            tc::tmem_ld16(lane_base + 3 * kCols + c0, v3);
            tc::tmem_wait_ld();
            const int comp = c0 >> 6;
            const bool store = rowok && !(comp == 1 && m == 0);
            const long long rowidx =
                comp == 0 ? ((long long)m * L1 + l) : ((L1 - m) * L1 + (l - m));
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int c = c0 + j;
              const int k = g * kGroupMaps + (c & 63);
              if (store && k < a.kc) {
                // levels 0 and 1 are exact integers: their weighted sum is exact in
                // FP32 as a (hi, lo) pair; levels 2 and 3 only touch lo.
                const float L0 = __uint_as_float(v0[j]);
                const float L1f = __uint_as_float(v1[j]) * 0x1p-8f;
                const float hi = L0 + L1f;
                const float bv = hi - L0;
                const float lo = ((L0 - (hi - bv)) + (L1f - bv)) +
                                 (__uint_as_float(v2[j]) * 0x1p-16f +
                                  __uint_as_float(v3[j]) * 0x1p-24f);
                const double v = ((double)hi + (double)lo) * rs * s_cs[c];
                double* dst = a.alm + rowidx * a.ld + a.k0 + k;
                if (a.nkc > 1) atomicAdd(dst, v);
                else if (a.accumulate) *dst += v;
                else *dst = v;
              }
            }
          }
        }
        tc::tc_fence_before();
        tc::mbar_arrive(&h.tempty);
      }
      ++tile_cnt;
      if (*abort) break;
    }
    __syncthreads();
    if (*abort) break;
  }
  // drain: the UMMA issuer waits for its last products before TMEM is released, and
  // the loader for its last copies
  if (tid == 160) {
    tc::umma_commit(&h.fin);
    for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
      if (tc::mbar_try_wait(&h.fin, 0)) break;
  }
  if (tid == 128) {
    for (uint32_t d = 0; d < (uint32_t)kStages && d < q_load; ++d) {
      const uint32_t q = q_load - 1 - d;
      for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
        if (tc::mbar_try_wait(&h.bfull[q % kStages], (q / kStages) & 1)) break;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (tid == 0 && h.abort) atomicOr(a.err, 1);
}

}  // namespace

size_t fsht_split_ws_bytes(int lmax, int nnorth, int kc) {
  const int ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  const int nks_max = (nnorth + kKStep - 1) / kKStep;
  return (size_t)(lmax + 1) * 2 * ngroups * nks_max * kSlices * kBTileBytes;
}
size_t fsht_split_eb_bytes(int lmax, int kc) {
  const int ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  return (size_t)(lmax + 1) * 2 * ngroups * kCols * sizeof(int);
}

int fsht_launch_split_prepare(fsht_plan* p, const double2* W, unsigned char* WS, int* EB,
                              double* alm, int nmaps_total, int k0, int kc, int accumulate,
                              cudaStream_t s) {
  const int ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  const int nks_max = (p->nnorth + kKStep - 1) / kKStep;
  const int nkc = (p->nnorth + kKChunk - 1) / kKChunk;
  SliceArgs sa;
  sa.W = W;
  sa.kc = kc;
  sa.nnorth = p->nnorth;
  sa.ngroups = ngroups;
  sa.nks_max = nks_max;
  sa.ring_i0 = p->d_ring_i0;
  sa.WS = WS;
  sa.EB = EB;
  k_slice_phase<<<dim3(p->lmax + 1, 2, ngroups), 128, 0, s>>>(sa);
  FSHT_LAUNCH_CHECK();
  if (nkc > 1 && !accumulate) {
    // K-chunks add into alm: clear this chunk's columns first
    const size_t L1 = (size_t)p->lmax + 1;
    FSHT_CUDA_TRY(cudaMemset2DAsync(alm + k0, sizeof(double) * nmaps_total, 0,
                                    sizeof(double) * kc, L1 * L1, s));
  }
  return FSHT_OK;
}

int fsht_launch_analysis_split(fsht_plan* p, const unsigned char* WS, const int* EB, double* alm,
                               int nmaps_total, int k0, int kc, int accumulate, cudaStream_t s) {
  const int ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  const int nks_max = (p->nnorth + kKStep - 1) / kKStep;
  const int nkc = (p->nnorth + kKChunk - 1) / kKChunk;
  SplitArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.ngroups = ngroups;
  a.nks_max = nks_max;
  a.nkc = nkc;
  a.cth = p->d_cth;
  a.sth = p->d_sth;
  a.pref = p->d_pref;
  a.ring_i0 = p->d_ring_i0;
  a.WS = WS;
  a.EB = EB;
  a.alm = alm;
  a.ld = nmaps_total;
  a.k0 = k0;
  a.kc = kc;
  a.pa = p->pa;
  a.accumulate = accumulate;
  a.err = p->d_err;
  const size_t sm = kABufBytes + kStages * kBStageBytes + (size_t)kKChunk * 20 + 1024;
  FSHT_CUDA_TRY(cudaFuncSetAttribute(k_analysis_split, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sm));
  const int npair = (p->lmax + 2) / 2;
  k_analysis_split<<<dim3(npair, 2 * nkc, ngroups), kThreads, sm, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}
