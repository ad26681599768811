// Split-precision Legendre analysis on the 5th-generation tensor cores (tcgen05).
//
// The precision form of the reference's per-m analysis contraction (get_plm_recursive
// + mat2alm, src/get_plm_recursive.f90:17-98, src/sht_core.f90:30-89):
//   a_lm = pa sum_i lambda_lm(theta_i) P_m(i),  P = S (l-m even) or D (l-m odd).
// Both operands are written as four balanced base-256 digits against power-of-two
// scales (rows of lambda: 2^EA(l) from the |Y_lm| bound; columns of P: 2^EB from the
// column maximum).  Digits are integers (|d0| <= 64, |d1..3| <= 128) that BF16 holds
// exactly, so every UMMA product is an exact integer.  The ten digit products of level
// a+b <= 3 run as BF16 UMMAs with FP32 accumulation, one TMEM accumulator per level:
//   level 0 and level 1 sums stay below 2^24 over <= 1024 rings, so they are exact
//   (a tile with more rings is accumulated in parts of <= 1024, each drained and added);
//   levels 2 and 3 carry weights 2^-16 and 2^-24, so FP32 rounding there is far
//   below the ~2^-31 representation error.
// The epilogue drains TMEM as FP32 (hi, lo) pairs (the levels joined on the FP32 pipe), hands
// it back to the UMMA issuer, and then applies the scales with one FP64 addition per element
// (pair_scaled).
//
// Three kernels per wave of m:
//   k_slice_phase    P -> digit tiles WS and column exponents EB (per 64-map group);
//   k_lambda_digits  the exponent-rescaled recursion in df64, once per (m, ring) for all
//                    map groups, written as lambda digit tiles into a staging buffer that
//                    holds one wave of m (a few GB at most: no P_lm table is kept);
//   k_split_gemm     persistent, one CTA per SM walking 128 x 128 output tiles, both
//                    operands streamed by bulk async copies (TMA engine) into a 6-stage
//                    ring, UMMAs into TMEM, eight epilogue warps.
// The synthesis counterparts (k_slice_alm, k_lambda_digits_T, k_split_synth) follow below.
// Max relative alm error against FP64: ~3e-8 (tests/test_gpu_split.py).
#include "split_common.cuh"

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

namespace {

// ------------------------------------------------------------------ P digits
// grid (m, parity, group), 128 threads = columns (map = c & 63, Re/Im = c >> 6).
// WS tile (m, p, g, t, digit): 128 columns x 16 rings, core matrices (8 cols x 8
// rings, 128 B) at (c/8)*256 + (k/8)*128.  Rings beyond the kept range are zero.
struct SliceArgs {
  const double* W;       // {S, D} as doubles: [m][ring][map][S|D][Re|Im]
  int kc, nnorth, ngroups, q0, lmax;
  size_t row_bytes;      // WS bytes per (wave-local q, parity, group)
  const int* ring_i0;
  unsigned char* WS;
  int* EB;
  int* err;              // plan error word (kErrRange when a value misses its scale)
};

// grid (q in wave, 4 x group), 128 threads = (ring half, map, parity, Re/Im) over one quarter
// (16 maps) of a 64-map group, Re/Im fastest, so a warp reads 8 maps' whole 32-byte {S, D}
// entries of one ring: every W sector is read once per pass (two passes: the column maximum,
// then the digits).  The two halves of a column's k-steps go to two threads (shorter serial
// chains, twice the loads in flight); their maxima meet in shared memory.  128 threads at <= 85
// registers (72 used: 9 K) fit in the register file beside the persistent contraction of the
// previous wave, whose 320 threads hold 168 registers each.
constexpr int kSliceThreads = 128;
__global__ void __launch_bounds__(kSliceThreads, 6) k_slice_phase(SliceArgs a) {
  __shared__ unsigned long long s_mx[kSliceThreads / 2];
  const int qi = blockIdx.x, g = blockIdx.y >> 2;
  const int m = m_of_q(a.q0 + qi, a.lmax);
  const int t = threadIdx.x & (kSliceThreads / 2 - 1), half = threadIdx.x / (kSliceThreads / 2);
  const int comp = t & 1, p = (t >> 1) & 1, kl = (t >> 2) + 16 * (blockIdx.y & 3);
  const int k = g * kGroupMaps + kl;
  const int c = comp * kGroupMaps + kl;
  const int i0 = a.ring_i0[m];
  const int K = a.nnorth - i0;
  const int nks = (K + kKStep - 1) / kKStep;
  const int ksh = (nks + 1) / 2;                   // k-steps of the first half
  const int ks_begin = half ? ksh : 0, ks_end = half ? nks : ksh;
  const int r_begin = ks_begin * kKStep, r_end = min(K, ks_end * kKStep);
  const bool valid = k < a.kc;
  const double* col = a.W + ((((long long)m * a.nnorth + i0) * a.kc + k) * 2 + p) * 2 + comp;
  const long long rstride = (long long)a.kc * 4;
  auto val = [&](int r) -> double { return (valid && r < K) ? col[r * rstride] : 0.0; };
  // The column maximum as FP64 bits with the sign cleared: for finite values the unsigned
  // integer order is the magnitude order, so the maximum takes integer operations only (an FP64
  // max runs on GB300's FP64 pipe at two per clock per SM, which bound this pass).
  constexpr unsigned long long kAbs = 0x7FFFFFFFFFFFFFFFull;
  unsigned long long mx = 0;
  if (valid) {
    // eight independent loads in flight per thread
    int r = r_begin;
    for (; r + 8 <= r_end; r += 8) {
      unsigned long long v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        v[u] = (unsigned long long)__double_as_longlong(col[(long long)(r + u) * rstride]) & kAbs;
#pragma unroll
      for (int u = 0; u < 8; ++u) mx = max(mx, v[u]);
    }
    for (; r < r_end; ++r)
      mx = max(mx, (unsigned long long)__double_as_longlong(col[(long long)r * rstride]) & kAbs);
  }
  if (half) s_mx[t] = mx;
  __syncthreads();
  if (!half) s_mx[t] = max(mx, s_mx[t]);
  __syncthreads();
  mx = s_mx[t];
  // |v| < 2^E for every value of the column (a subnormal maximum takes E = -1021; a
  // non-finite one gives an exponent its digits report as out of range)
  const int ef = (int)(mx >> 52);
  const int E = mx == 0 ? kEmptyExp : (ef == 0 ? -1021 : ef - 1022);
  if (!half) a.EB[(((long long)qi * 2 + p) * a.ngroups + g) * kCols + c] = E;
  unsigned char* base = a.WS + ((size_t)(qi * 2 + p) * a.ngroups + g) * a.row_bytes +
                        (c >> 3) * 256 + (c & 7) * 16;
  bool bad = false;
  for (int ts = ks_begin; ts < ks_end; ++ts) {
    // the k-step's 16 loads issued together (the column is not in L2 any more)
    double v[kKStep];
#pragma unroll
    for (int u = 0; u < kKStep; ++u) v[u] = val(ts * kKStep + u);
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      uint16_t sl[kSlices][8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        uint16_t q4[4] = {0, 0, 0, 0};
        if (E != kEmptyExp) bad |= tc::digits4_f(v[hh * 8 + j], E, q4);
        for (int d = 0; d < kSlices; ++d) sl[d][j] = q4[d];
      }
      for (int d = 0; d < kSlices; ++d) {
        uint4 pk;
        pk.x = sl[d][0] | ((uint32_t)sl[d][1] << 16);
        pk.y = sl[d][2] | ((uint32_t)sl[d][3] << 16);
        pk.z = sl[d][4] | ((uint32_t)sl[d][5] << 16);
        pk.w = sl[d][6] | ((uint32_t)sl[d][7] << 16);
        *reinterpret_cast<uint4*>(base + ((size_t)ts * kSlices + d) * kBTileBytes + hh * 128) = pk;
      }
    }
  }
  if (bad) atomicOr(a.err, tc::kErrRange);
}

// ------------------------------------------------------------------ lambda digits
// Scaled recursion.  With D_l = prod_{k=m+1..l} a_k (D_m = 1) and mu_l = lambda_l / D_l:
//   mu_l = x mu_{l-1} - beta_l mu_{l-2},   beta_l = b_l / (a_l a_{l-1})   (beta_{m+1} = 0),
// two FP64 operations per step instead of four.  Rows are digitised as
// lambda_l / Dm_l = mu 2^(Et + Dx_l) against 2^EA(l) with EA(l) from |lambda| / Dm_l <=
// sqrt((2l+1)/4pi) / Dm_l (D_l = Dm_l 2^Dx_l, Dm_l in [1, 2)); the GEMM epilogue multiplies
// row l by Dm_l 2^EA(l).  Et is the per-ring exponent carried with the state.
// One thread per m, sequential in l: beta_l, Dm_l, Dx_l and erow_l = EA(l) - Dx_l.
__global__ void k_lam_table(int lmax, FshtLamRow* tab) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m > lmax) return;
  FshtLamRow* row = tab + tri_off(m, lmax);
  double dm = 1.0, a_prev = 0.0;
  int dx = 0;
  for (int l = m; l <= lmax; ++l) {
    double beta = 0.0;
    if (l > m) {
      const RecConst c = rec_coeffs(l, m);
      beta = (l == m + 1) ? 0.0 : c.b / (c.a * a_prev);
      int t;
      dm = frexp(dm * c.a, &t);     // [0.5, 1)
      dm *= 2.0;
      dx += t - 1;
      a_prev = c.a;
    }
    const double bound = sqrt((2.0 * l + 1.0) / (4.0 * M_PI)) * (1.0 + 0x1p-30) / dm;
    const int ea = ilogb(bound) + 1;
    FshtLamRow r;
    r.beta = beta;
    r.dm = dm;
    r.erow = ea - dx;
    r.dx = dx;
    row[l - m] = r;
  }
}

// grid (q in wave, 128-ring block), 128 threads = rings.  Writes the four digit tiles of
// every (parity, l-tile, k-step) the block covers, in the UMMA K-major core-matrix layout
// (core matrix 8 rows x 8 rings, 128 B, at (row/8)*256 + (ring/8)*128 within a 4 KB tile).
struct LamArgs {
  int lmax, nnorth, q0;
  const double* cth;
  const double* sth;
  const double* pref;
  const int* ring_i0;
  const FshtLamRow* tab;
  const long long* lam_off;
  unsigned char* lbuf;
  int* err;
};

constexpr int kLamBlock = 32;                 // l per staging block (16 rows per parity)
constexpr int kStageStride = kSCRings + 2;    // uint64 per staged row (+16 B against conflicts)

__global__ void __launch_bounds__(128) k_lambda_digits(LamArgs a) {
  __shared__ __align__(16) unsigned long long S[2][kLamBlock / 2][kStageStride];
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
  unsigned char* base = a.lbuf + (size_t)(a.lam_off[q] - a.lam_off[a.q0]) * kSlices * kATileBytes;
  const FshtLamRow* tab = a.tab + tri_off(m, a.lmax);

  // The recursion runs in df64 (FP32 pairs, ~48 significand bits) on the FP32 pipe: the
  // digits need 2^-31 of each row's scale and the recursion's error stays near l 2^-48, while
  // GB300's FP64 pipe (two operations per clock per SM) would bound this kernel.  The state
  // (s1, s2) = (mu_l, mu_{l-1}) 2^-et is kept within 2^-32 .. 2^32 after every step: one step
  // changes max(|s1|, |s2|) by at most a factor 2 up and beta / 2 >= 2^-14 down, so FP32
  // exponents (and the low parts, 2^24 below) never leave the normal range.
  float xh = 0.f, xl = 0.f, s1h = 0.f, s1l = 0.f, s2h = 0.f, s2l = 0.f;
  int et = 0;
  if (valid) {
    int e, k;
    const double x = a.cth[i0 + r];
    double s1;
    rec_seed(a.sth[i0 + r], a.pref[m], m, s1, e);
    const double f = frexp(s1, &k);           // s1 = f 2^k, |f| in [0.5, 1)
    et = 600 * e + k;
    s1h = __double2float_rn(f);
    s1l = __double2float_rn(f - (double)s1h);
    xh = __double2float_rn(x);
    xl = __double2float_rn(x - (double)xh);
  }
  // the 32 recursion rows of the current block, staged in shared memory (uniform reads
  // off the dependency chain): -beta as a df64 pair
  __shared__ float2 s_beta[kLamBlock];
  __shared__ int s_erow[kLamBlock];
  if (tid < kLamBlock && m + tid <= a.lmax) {
    const double b = tab[tid].beta;
    const float bh = __double2float_rn(b);
    s_beta[tid] = make_float2(-bh, -__double2float_rn(b - (double)bh));
    s_erow[tid] = tab[tid].erow;
  }
  __syncthreads();
  const int lend = ntiles * 2 * kRows;
  bool bad = false;
  for (int lb = 0; lb < lend; lb += kLamBlock) {
#pragma unroll 4
    for (int jj = 0; jj < kLamBlock; ++jj) {
      const int j = lb + jj;
      unsigned long long pk = 0;
      if (m + j <= a.lmax) {
        const float2 nb = s_beta[jj];
        const int erow = s_erow[jj];
        if (j > 0) {
          float nh, nl;
          dd::dot2(xh, xl, s1h, s1l, nb.x, nb.y, s2h, s2l, nh, nl);   // x mu1 - beta mu2
          s2h = s1h;
          s2l = s1l;
          s1h = nh;
          s1l = nl;
          const float am = fmaxf(fabsf(s1h), fabsf(s2h));
          if (am > 0x1p32f) {
            s1h *= 0x1p-64f; s1l *= 0x1p-64f; s2h *= 0x1p-64f; s2l *= 0x1p-64f;
            et += 64;
          } else if (am < 0x1p-32f && am > 0.f) {
            s1h *= 0x1p64f; s1l *= 0x1p64f; s2h *= 0x1p64f; s2l *= 0x1p64f;
            et -= 64;
          }
        }
        if (valid) {
          uint16_t d[4];
          bad |= tc::digits4_df(s1h, s1l, erow - et, d);
          pk = (unsigned long long)d[0] | ((unsigned long long)d[1] << 16) |
               ((unsigned long long)d[2] << 32) | ((unsigned long long)d[3] << 48);
        }
      }
      S[jj & 1][jj >> 1][tid] = pk;
    }
    __syncthreads();
    // write-out: unit u = (r8: 3 bits, khalf, rg, ks: 3 bits, parity); a warp stores 512
    // contiguous bytes of one digit tile per instruction
    const int t = lb / (2 * kRows);
    const int rowt0 = (lb % (2 * kRows)) >> 1;
    for (int u = tid; u < 2 * (kLamBlock / 2) * (kSCRings / 8); u += 128) {
      const int r8 = u & 7, khalf = (u >> 3) & 1, rg = (u >> 4) & 1, ks = (u >> 5) & 7,
                p = u >> 8;
      const int gks = rb * (kSCRings / kKStep) + ks;
      if (gks >= nks) continue;
      const int row = rg * 8 + r8;
      const unsigned long long* src = &S[p][row][ks * kKStep + khalf * 8];
      unsigned long long v[8];
#pragma unroll
      for (int i = 0; i < 8; i += 2) {
        const ulonglong2 w = *reinterpret_cast<const ulonglong2*>(src + i);
        v[i] = w.x;
        v[i + 1] = w.y;
      }
      const int rowt = rowt0 + row;
      unsigned char* tile =
          base + ((size_t)(p * ntiles + t) * nks + gks) * kSlices * kATileBytes +
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
    if (tid < kLamBlock && m + lb + kLamBlock + tid <= a.lmax) {
      const double b = tab[lb + kLamBlock + tid].beta;
      const float bh = __double2float_rn(b);
      s_beta[tid] = make_float2(-bh, -__double2float_rn(b - (double)bh));
      s_erow[tid] = tab[lb + kLamBlock + tid].erow;
    }
    __syncthreads();
  }
  if (bad) atomicOr(a.err, tc::kErrRange);
}

// ------------------------------------------------------------------ split GEMM
// Persistent: one CTA per SM walks the wave's work units u = blockIdx.x, + gridDim.x, ...;
// a unit is (q, parity, l-tile, 64-map group), the group fastest, so CTAs running at the same
// time share lambda tiles in L2.  A unit is one 128-row x 128-column output tile over all of
// its k-steps of 16 rings, accumulated in parts of <= 64 k-steps (1024 rings keep levels 0
// and 1 exact in FP32): the first part's epilogue stores, later parts add as fire-and-forget
// reductions (one thread owns each element, so the result is deterministic).  Warp 8 lane 0 streams lambda and P digit tiles (bulk async copies) through a
// kStagesG-deep ring that runs on across parts and units, so the next tiles load while an
// epilogue drains the accumulators; warp 9 lane 0 issues the ten level-ordered UMMAs per
// k-step; warps 0-7 run the epilogue.  TMEM (four 128-column level accumulators) is
// allocated once per CTA; tfull / tempty hand it between the UMMA issuer and the epilogue for
// every part.
constexpr int kStagesG = 6;
constexpr uint32_t kStageBytesG = 2 * kSlices * kATileBytes;    // 32 KB: A then B
constexpr int kPartSteps = kKChunk / kKStep;   // most k-steps per part (levels 0, 1 exact)
constexpr size_t kSmemG = (size_t)kStagesG * kStageBytesG + kStgBytes;

struct GemmArgs {
  int lmax, nnorth, ngroups, q0, ntmax, accumulate, nunits;
  int part_steps;        // k-steps per ring part, <= kPartSteps (the plan's tile choice)
  size_t row_bytes;
  const int* ring_i0;
  const long long* lam_off;
  const FshtLamRow* tab;
  const unsigned char* lbuf;
  const unsigned char* WS;
  const int* EB;
  double* alm;
  int ld, k0, kc;
  double pa;
  int* err;
};

struct __align__(8) GemmSmemHdr {
  uint64_t full[kStagesG], empty[kStagesG], tfull, tempty, fin;
  uint32_t tmem;
  int abort;
};

// One work unit, decoded from its index; nks = 0: nothing to do (l-tile beyond lmax - m).
struct GemmUnit {
  int g, p, t, qi, m, nks, ntiles, lt0;
};

__device__ __forceinline__ GemmUnit gemm_unit(const GemmArgs& a, int u) {
  GemmUnit w;
  w.g = u % a.ngroups;
  int r = u / a.ngroups;
  w.p = r & 1;
  r >>= 1;
  w.t = r % a.ntmax;
  w.qi = r / a.ntmax;
  w.m = m_of_q(a.q0 + w.qi, a.lmax);
  const int K = a.nnorth - a.ring_i0[w.m];
  w.ntiles = (a.lmax - w.m + 1 + 2 * kRows - 1) / (2 * kRows);
  w.nks = w.t < w.ntiles ? (K + kKStep - 1) / kKStep : 0;
  w.lt0 = w.m + w.t * 2 * kRows;
  return w;
}

__global__ void __launch_bounds__(kThreadsG, 1) k_split_gemm(GemmArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ GemmSmemHdr h;
  __shared__ int s_ce[kCols];          // column exponents (eb - 12) of the current unit

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  volatile int* abort = &h.abort;
  if (tid == 0) {
    for (int s = 0; s < kStagesG; ++s) {
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
    // producer: the k-step ring runs on across parts and units
    uint32_t i = 0;
    for (int u = blockIdx.x; u < a.nunits && !*abort; u += gridDim.x) {
      const GemmUnit w = gemm_unit(a, u);
      if (w.nks == 0) continue;
      const unsigned char* asrc =
          a.lbuf + (size_t)(a.lam_off[a.q0 + w.qi] - a.lam_off[a.q0]) * kSlices * kATileBytes +
          (size_t)(w.p * w.ntiles + w.t) * w.nks * kSlices * kATileBytes;
      const unsigned char* bsrc =
          a.WS + (((size_t)w.qi * 2 + w.p) * a.ngroups + w.g) * a.row_bytes;
      bool ok = true;
      for (int k = 0; k < w.nks; ++k, ++i) {
        const uint32_t st = i % kStagesG;
        if (!tc::mbar_wait(&h.empty[st], ((i / kStagesG) & 1) ^ 1, abort)) {
          ok = false;
          break;
        }
        unsigned char* dst = smem + st * kStageBytesG;
        tc::mbar_arrive_expect_tx(&h.full[st], kStageBytesG);
        tc::bulk_g2s(dst, asrc + (size_t)k * kSlices * kATileBytes, kSlices * kATileBytes,
                     &h.full[st]);
        tc::bulk_g2s(dst + kSlices * kATileBytes, bsrc + (size_t)k * kSlices * kBTileBytes,
                     kSlices * kBTileBytes, &h.full[st]);
        ++n_loaded;
      }
      if (!ok) break;
    }
  } else if (tid == kEpiThreads + 32) {
    // UMMA issuer
    const uint32_t idesc = tc::umma_idesc_bf16(kRows, kCols);
    const uint32_t s_u = tc::smem_u32(smem);
    uint32_t i = 0, np = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < a.nunits && ok && !*abort; u += gridDim.x) {
      const GemmUnit w = gemm_unit(a, u);
      for (int ks0 = 0; ks0 < w.nks && ok; ks0 += a.part_steps, ++np) {
        // the epilogue of the previous part has read the accumulators
        if (np > 0 && !tc::mbar_wait(&h.tempty, (np - 1) & 1, abort)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const int nk = min(w.nks - ks0, a.part_steps);
        for (int k = 0; k < nk; ++k, ++i) {
          const uint32_t st = i % kStagesG;
          if (!tc::mbar_wait(&h.full[st], (i / kStagesG) & 1, abort)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const uint32_t abase = s_u + st * kStageBytesG;
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
  } else if (tid < kEpiThreads) {
    // epilogue (warps 0-7): TMEM -> alm, row = TMEM lane (warp % 4 picks the lane quarter,
    // warp / 4 the half of the columns).  No early exit: the epilogue threads must meet at
    // every named barrier, so after an expired wait (abort) the remaining parts are walked
    // without work.
    const int lane = tid & 31;
    const int row0 = (warp & 3) << 5;              // this warp's 32 rows (its TMEM lane quarter)
    const int row = row0 + lane;
    const int cbeg = (warp >> 2) * (kCols / 2);   // this warp's half of the columns
    const int comp = cbeg >> 6;                    // Re (0) or Im (1) of its 64 maps
    const long long L1 = a.lmax + 1;
    const uint32_t lane_base = tmem + ((uint32_t)row0 << 16);
    double* stg = reinterpret_cast<double*>(smem + (size_t)kStagesG * kStageBytesG) +
                  (size_t)warp * kStgWarpDoubles;
    uint32_t np = 0;
    for (int u = blockIdx.x; u < a.nunits; u += gridDim.x) {
      const GemmUnit w = gemm_unit(a, u);
      if (w.nks == 0) continue;
      // this unit's column exponents and this thread's row factor
      {
        const int eb =
            tid < kCols ? a.EB[(((long long)w.qi * 2 + w.p) * a.ngroups + w.g) * kCols + tid] : 0;
        // the previous unit's readers of s_ce are done (named barrier of the epilogue threads)
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
        if (tid < kCols) s_ce[tid] = (eb == kEmptyExp) ? kEmptyExp : eb - 12;
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
      }
      const int l = w.lt0 + w.p + 2 * row;
      const bool rowok = l <= a.lmax;
      float rh = 0.f, rl = 0.f;
      int re = 0;
      if (rowok) {
        const FshtLamRow rw = a.tab[tri_off(w.m, a.lmax) + (l - w.m)];
        factor_pair(rw.dm * a.pa, rh, rl);
        re = rw.erow + rw.dx;
      }
      for (int ks0 = 0; ks0 < w.nks; ks0 += a.part_steps) {
        bool ok = tc::mbar_wait(&h.tfull, np & 1, abort);
        ok = __all_sync(0xffffffffu, ok);      // tcgen05.ld below is warp-collective
        ++np;
        if (!ok) continue;
        tc::tc_fence_after();
        const bool add = ks0 > 0 || a.accumulate;
        // Im of m = 0 does not exist
        const bool comp_ok = !(comp == 1 && w.m == 0);
        // Drain first: this lane's row of the warp's 64 columns leaves TMEM as FP32 (hi, lo)
        // pairs (the four levels joined exactly, FP32 pipe only, 128 registers) and TMEM goes
        // back to the UMMA issuer before any FP64 instruction or global store, so the next
        // part's products run under the rest of this epilogue (on GB300 the FP64 pipe does two
        // operations per clock per SM: the joining additions of a whole part take ~4 us).
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
          // this lane's row of the block, staged
#pragma unroll
          for (int j = 0; j < 16; ++j)
            stg[stg_at(lane, j)] =
                rowok ? pair_scaled(hh[cr + j], ll[cr + j], rh, rl, re + s_ce[c0 + j]) : 0.0;
          __syncwarp();
          // the block back out by rows: lanes 0-15 one row, 16-31 the next, 16 maps each.
          // Adds go out as fire-and-forget reductions (no load latency in the epilogue); one
          // thread owns each element within a part and parts are ordered by the TMEM hand-over,
          // so the order (store, then adds) is fixed and the result is deterministic.
          const int cc = lane & 15;
          const int k = w.g * kGroupMaps + ((c0 + cc) & 63);
          if (comp_ok && k < a.kc) {
#pragma unroll 4
            for (int i = 0; i < 16; ++i) {
              const int r = 2 * i + (lane >> 4);
              const int lr = w.lt0 + w.p + 2 * (row0 + r);
              if (lr <= a.lmax) {
                const long long rowidx =
                    comp == 0 ? ((long long)w.m * L1 + lr) : ((L1 - w.m) * L1 + (lr - w.m));
                double* dst = a.alm + rowidx * a.ld + a.k0 + k;
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
  // drain: the UMMA issuer waits for its last products before TMEM is released, and the
  // loader for its last copies
  if (tid == kEpiThreads + 32) {
    tc::umma_commit(&h.fin);
    for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
      if (tc::mbar_try_wait(&h.fin, 0)) break;
  }
  if (tid == kEpiThreads) {
    for (uint32_t d = 0; d < (uint32_t)kStagesG && d < n_loaded; ++d) {
      const uint32_t i = n_loaded - 1 - d;
      for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
        if (tc::mbar_try_wait(&h.full[i % kStagesG], (i / kStagesG) & 1)) break;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (tid == 0 && h.abort) atomicOr(a.err, tc::kErrTimeout);
}


// ------------------------------------------------------------------ synthesis
// G_m(i) = sum_l a_lm lambda_lm(theta_i) as even-l and odd-l parts E, O (G_N = E + O,
// G_S = E - O).  GEMM per (m, parity): D[ring][col] = sum_l lambda[l][ring] a[l][col] with
// K = l.  A scale must not depend on the summation index, so lambda is digitised against
// one global 2^EAG (EAG from sqrt((2 lmax + 1)/4pi)) as lambda = mu Dm 2^(Et + Dx): one more
// FP64 multiply per step than the analysis tiles.  Tiles: 128 rings x 16 l of one parity,
// K-major (core matrix 8 rings x 8 l at (ring/8)*256 + (l/8)*128).

// grid (q in wave, 128-ring block), 128 threads = rings; every thread stores its own
// 16-byte core-matrix rows (8 l of one parity), no staging.
struct LamTArgs {
  int lmax, nnorth, q0, eag;
  const double* cth;
  const double* sth;
  const double* pref;
  const int* ring_i0;
  const FshtLamRow* tab;
  const long long* lam_offT;
  unsigned char* lbuf;
  int* err;
};

__global__ void __launch_bounds__(128) k_lambda_digits_T(LamTArgs a) {
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
      a.lbuf + (size_t)(a.lam_offT[q] - a.lam_offT[a.q0]) * kSlices * kATileBytes +
      (tid >> 3) * 256 + (tid & 7) * 16;
  const FshtLamRow* tab = a.tab + tri_off(m, a.lmax);
  // df64 recursion with per-step rescaling, as in k_lambda_digits
  float xh = 0.f, xl = 0.f, s1h = 0.f, s1l = 0.f, s2h = 0.f, s2l = 0.f;
  int et = 0;
  if (valid) {
    int e, kx;
    const double x = a.cth[i0 + r];
    double s1;
    rec_seed(a.sth[i0 + r], a.pref[m], m, s1, e);
    const double f = frexp(s1, &kx);
    et = 600 * e + kx;
    s1h = __double2float_rn(f);
    s1l = __double2float_rn(f - (double)s1h);
    xh = __double2float_rn(x);
    xl = __double2float_rn(x - (double)xh);
  }
  __shared__ float4 s_bd[32];             // (-beta, Dm) as df64 pairs
  __shared__ int s_dx[32];
  bool bad = false;
  for (int kl = 0; kl < nkl; ++kl) {
    __syncthreads();                      // the previous block's rows are no longer read
    if (tid < 32 && m + kl * 32 + tid <= a.lmax) {
      const FshtLamRow rw = tab[kl * 32 + tid];
      const float bh = __double2float_rn(rw.beta), dh = __double2float_rn(rw.dm);
      s_bd[tid] = make_float4(-bh, -__double2float_rn(rw.beta - (double)bh), dh,
                              __double2float_rn(rw.dm - (double)dh));
      s_dx[tid] = rw.dx;
    }
    __syncthreads();
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      uint32_t pk[2][kSlices][4];
#pragma unroll
      for (int pp = 0; pp < 2; ++pp)
#pragma unroll
        for (int d = 0; d < kSlices; ++d)
#pragma unroll
          for (int w = 0; w < 4; ++w) pk[pp][d][w] = 0;
#pragma unroll
      for (int jj = 0; jj < 16; ++jj) {
        const int j = kl * 32 + half * 16 + jj;
        uint16_t d[4] = {0, 0, 0, 0};
        if (m + j <= a.lmax) {
          const float4 bd = s_bd[half * 16 + jj];
          if (j > 0) {
            float nh, nl;
            dd::dot2(xh, xl, s1h, s1l, bd.x, bd.y, s2h, s2l, nh, nl);   // x mu1 - beta mu2
            s2h = s1h;
            s2l = s1l;
            s1h = nh;
            s1l = nl;
            const float am = fmaxf(fabsf(s1h), fabsf(s2h));
            if (am > 0x1p32f) {
              s1h *= 0x1p-64f; s1l *= 0x1p-64f; s2h *= 0x1p-64f; s2l *= 0x1p-64f;
              et += 64;
            } else if (am < 0x1p-32f && am > 0.f) {
              s1h *= 0x1p64f; s1l *= 0x1p64f; s2h *= 0x1p64f; s2l *= 0x1p64f;
              et -= 64;
            }
          }
          if (valid) {
            float vh, vl;
            dd::mul(s1h, s1l, bd.z, bd.w, vh, vl);                     // mu Dm
            bad |= tc::digits4_df(vh, vl, a.eag - et - s_dx[half * 16 + jj], d);
          }
        }
        const int par = jj & 1, slot = jj >> 1;
#pragma unroll
        for (int dd = 0; dd < kSlices; ++dd)
          pk[par][dd][slot >> 1] |= (uint32_t)d[dd] << (16 * (slot & 1));
      }
#pragma unroll
      for (int par = 0; par < 2; ++par)
#pragma unroll
        for (int dd = 0; dd < kSlices; ++dd) {
          uint4 o;
          o.x = pk[par][dd][0];
          o.y = pk[par][dd][1];
          o.z = pk[par][dd][2];
          o.w = pk[par][dd][3];
          *reinterpret_cast<uint4*>(
              base + (((size_t)(par * nrb + rb) * nkl + kl) * kSlices + dd) * kATileBytes +
              half * 128) = o;
        }
    }
  }
  if (bad) atomicOr(a.err, tc::kErrRange);
}

// alm -> digit tiles: grid (m, parity, group), 128 threads = columns (map = c & 63,
// Re/Im = c >> 6).  Tile (m, p, g, l-step): 128 columns x 16 l, K-major.
struct SliceAArgs {
  const double* alm;
  int ld, k0, kc, lmax, ngroups, q0;
  size_t row_bytes;
  unsigned char* WS;
  int* EB;
  int* err;
};

__global__ void __launch_bounds__(128) k_slice_alm(SliceAArgs a) {
  const int qi = blockIdx.x, p = blockIdx.y, g = blockIdx.z;
  const int m = m_of_q(a.q0 + qi, a.lmax);
  const int c = threadIdx.x;
  const int k = g * kGroupMaps + (c & 63);
  const int comp = c >> 6;
  const bool valid = k < a.kc && !(comp == 1 && m == 0);
  const long long L1 = a.lmax + 1;
  const int cnt0 = (a.lmax - m) / 2 + 1;
  const int cnt = (p == 0) ? cnt0 : (a.lmax > m ? (a.lmax - m - 1) / 2 + 1 : 0);
  auto val = [&](int idx) -> double {
    if (!valid || idx >= cnt) return 0.0;
    const int l = m + p + 2 * idx;
    const long long row = comp == 0 ? (long long)m * L1 + l : (L1 - m) * L1 + (l - m);
    return a.alm[row * a.ld + a.k0 + k];
  };
  // column maximum on FP64 bits with the sign cleared (integer operations, as in
  // k_slice_phase)
  unsigned long long mx = 0;
  for (int idx = 0; idx < cnt; ++idx)
    mx = max(mx, (unsigned long long)__double_as_longlong(val(idx)) & 0x7FFFFFFFFFFFFFFFull);
  const int ef = (int)(mx >> 52);
  const int E = mx == 0 ? kEmptyExp : (ef == 0 ? -1021 : ef - 1022);
  a.EB[(((long long)qi * 2 + p) * a.ngroups + g) * kCols + c] = E;
  const int nkl = (cnt0 + kKStep - 1) / kKStep;
  unsigned char* base = a.WS +
                        ((size_t)(qi * 2 + p) * a.ngroups + g) * a.row_bytes +
                        (c >> 3) * 256 + (c & 7) * 16;
  bool bad = false;
  for (int kl = 0; kl < nkl; ++kl) {
    for (int half = 0; half < 2; ++half) {
      uint16_t sl[kSynthPlanes][8];
      for (int j = 0; j < 8; ++j) {
        uint16_t q4[4] = {0, 0, 0, 0};
        if (E != kEmptyExp) bad |= tc::digits4_f(val(kl * kKStep + half * 8 + j), E, q4);
        for (int d = 0; d < kSlices; ++d) sl[d][j] = q4[d];
        for (int d = 1; d < kSlices; ++d) sl[kSlices - 1 + d][j] = tc::bf16_scale_2m8(q4[d]);
      }
      for (int d = 0; d < kSynthPlanes; ++d) {
        uint4 pk;
        pk.x = sl[d][0] | ((uint32_t)sl[d][1] << 16);
        pk.y = sl[d][2] | ((uint32_t)sl[d][3] << 16);
        pk.z = sl[d][4] | ((uint32_t)sl[d][5] << 16);
        pk.w = sl[d][6] | ((uint32_t)sl[d][7] << 16);
        *reinterpret_cast<uint4*>(base + (size_t)kl * kSynthBBytes + (size_t)d * kBTileBytes +
                                  half * 128) = pk;
      }
    }
  }
  if (bad) atomicOr(a.err, tc::kErrRange);
}

// CTA = (64-map group, 128-ring block x l-chunk, q): both parities in turn through the same
// TMEM accumulators (E first, written as G_N = G_S = E; then O, added to G_N and subtracted
// from G_S by the same threads).  Roles as in k_split_gemm.
struct SynthArgs {
  int lmax, nnorth, ngroups, q0, nrbmax, eag, nunits;
  size_t row_bytes;
  const int* ring_i0;
  const long long* lam_offT;
  const unsigned char* lbuf;
  const unsigned char* WS;
  const int* EB;
  double* W;           // double2 {G_N, G_S} as doubles
  int kc;
  int* err;
};

constexpr int kStagesS = 4;
constexpr uint32_t kStageBytesS = kSlices * kATileBytes + kSynthBBytes;   // 44 KB
constexpr int kPartStepsS = kKChunk / kKStep;

struct __align__(8) SynthSmemHdr {
  uint64_t full[kStagesS], empty[kStagesS], tfull, tempty, fin;
  uint32_t tmem;
  int abort;
};

// One work unit (q, 128-ring block, 64-map group), the group fastest; nkl = 0: nothing to do.
struct SynthUnit {
  int g, rb, qi, m, i0, K, nrb, nkl;
};

__device__ __forceinline__ SynthUnit synth_unit(const SynthArgs& a, int u) {
  SynthUnit w;
  w.g = u % a.ngroups;
  int r = u / a.ngroups;
  w.rb = r % a.nrbmax;
  w.qi = r / a.nrbmax;
  w.m = m_of_q(a.q0 + w.qi, a.lmax);
  w.i0 = a.ring_i0[w.m];
  w.K = a.nnorth - w.i0;
  w.nrb = (w.K + kSCRings - 1) / kSCRings;
  w.nkl = w.rb < w.nrb ? ((a.lmax - w.m) / 2 + 1 + kKStep - 1) / kKStep : 0;
  return w;
}

// Persistent like k_split_gemm: one CTA per SM walks the units; per part of <= 64 l-steps
// (1024 l keep levels 0 and 1 exact) the even-l pass then the odd-l pass run through the same
// TMEM accumulators.  The first even pass of a unit writes G_N = G_S = E, every later pass adds
// (+E, or +O to G_N and -O to G_S) as fire-and-forget reductions from the thread that owns the
// element, so W needs no clearing and the result is deterministic.  Warps 0-7: epilogue (two
// per TMEM lane quarter, one per half of the columns), warp 8 lane 0: copies, warp 9 lane 0:
// UMMAs (13 per l-step: levels 0-3 and the level-4 fold).
__global__ void __launch_bounds__(kThreadsG, 1) k_split_synth(SynthArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ SynthSmemHdr h;
  __shared__ int s_ce[2][kCols];       // column exponents EAG + eb - 12 per parity

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  volatile int* abort = &h.abort;
  if (tid == 0) {
    for (int s = 0; s < kStagesS; ++s) {
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
      const SynthUnit w = synth_unit(a, u);
      if (w.nkl == 0) continue;
      const unsigned char* abase =
          a.lbuf + (size_t)(a.lam_offT[a.q0 + w.qi] - a.lam_offT[a.q0]) * kSlices * kATileBytes;
      for (int kl0 = 0; kl0 < w.nkl && ok; kl0 += kPartStepsS) {
        const int nk = min(w.nkl - kl0, kPartStepsS);
        for (int par = 0; par < 2 && ok; ++par) {
          for (int kk = kl0; kk < kl0 + nk; ++kk, ++i) {
            const uint32_t st = i % kStagesS;
            if (!tc::mbar_wait(&h.empty[st], ((i / kStagesS) & 1) ^ 1, abort)) {
              ok = false;
              break;
            }
            unsigned char* dst = smem + st * kStageBytesS;
            const unsigned char* asrc =
                abase + ((size_t)(par * w.nrb + w.rb) * w.nkl + kk) * kSlices * kATileBytes;
            const unsigned char* bsrc =
                a.WS + (((size_t)w.qi * 2 + par) * a.ngroups + w.g) * a.row_bytes +
                (size_t)kk * kSynthBBytes;
            tc::mbar_arrive_expect_tx(&h.full[st], kStageBytesS);
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
      const SynthUnit w = synth_unit(a, u);
      for (int kl0 = 0; kl0 < w.nkl && ok; kl0 += kPartStepsS) {
        const int nk = min(w.nkl - kl0, kPartStepsS);
        for (int par = 0; par < 2 && ok; ++par, ++np) {
          if (np > 0 && !tc::mbar_wait(&h.tempty, (np - 1) & 1, abort)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          for (int k = 0; k < nk; ++k, ++i) {
            const uint32_t st = i % kStagesS;
            if (!tc::mbar_wait(&h.full[st], (i / kStagesS) & 1, abort)) {
              ok = false;
              break;
            }
            tc::tc_fence_after();
            const uint32_t abase = s_u + st * kStageBytesS;
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
            // level 4 (a1 b3, a2 b2, a3 b1) into the level-3 accumulator via the 2^-8 planes:
            // with lambda against one scale its digits are often small, and dropping level 4
            // would cost ~2e-7
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
      const SynthUnit w = synth_unit(a, u);
      if (w.nkl == 0) continue;
      {
        int e[2] = {0, 0};
        if (tid < kCols)
          for (int pp = 0; pp < 2; ++pp)
            e[pp] = a.EB[(((long long)w.qi * 2 + pp) * a.ngroups + w.g) * kCols + tid];
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
        if (tid < kCols)
          for (int pp = 0; pp < 2; ++pp)
            s_ce[pp][tid] = (e[pp] == kEmptyExp) ? kEmptyExp : a.eag + e[pp] - 12;
        asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
      }
      const int rr = w.rb * kSCRings + row;
      const bool rowok = rr < w.K;
      const int i = w.i0 + rr;
      for (int kl0 = 0; kl0 < w.nkl; kl0 += kPartStepsS) {
        for (int par = 0; par < 2; ++par) {
          bool ok = tc::mbar_wait(&h.tfull, np & 1, abort);
          ok = __all_sync(0xffffffffu, ok);
          ++np;
          if (!ok) continue;
          tc::tc_fence_after();
          const bool first = kl0 == 0 && par == 0;
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
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int c = c0 + j;
              const int k = w.g * kGroupMaps + (c & 63);
              if (rowok && k < a.kc) {
                const double v =
                    levels_scaled(v0[j], v1[j], v2[j], v3[j], 1.f, 0.f, s_ce[par][c]);
                double* gn = a.W + ((((long long)w.m * a.nnorth + i) * a.kc + k) * 2) * 2 + comp;
                double* gs = gn + 2;
                if (first) {
                  *gn = v;
                  *gs = v;
                } else {
                  atomicAdd(gn, v);
                  atomicAdd(gs, par ? -v : v);
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
    for (uint32_t d = 0; d < (uint32_t)kStagesS && d < n_loaded; ++d) {
      const uint32_t i = n_loaded - 1 - d;
      for (uint32_t it = 0; it < tc::kWaitLimit; ++it)
        if (tc::mbar_try_wait(&h.full[i % kStagesS], (i / kStagesS) & 1)) break;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
  if (tid == 0 && h.abort) atomicOr(a.err, tc::kErrTimeout);
}

}  // namespace


// WS and EB hold one wave of m (the wave with the most orders).
size_t fsht_split_ws_bytes(const fsht_plan* p, int kc) {
  const int ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  return (size_t)p->wave_qmax * 2 * ngroups * ws_row_bytes(p->lmax, p->nnorth);
}
size_t fsht_split_eb_bytes(const fsht_plan* p, int kc) {
  const int ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  return (size_t)p->wave_qmax * 2 * ngroups * kCols * sizeof(int);
}

int fsht_launch_split_slice(fsht_plan* p, int w, const double2* W, unsigned char* WS, int* EB,
                            int kc, cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  SliceArgs sa;
  sa.W = reinterpret_cast<const double*>(W);
  sa.kc = kc;
  sa.nnorth = p->nnorth;
  sa.ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  sa.q0 = wv[0];
  sa.lmax = p->lmax;
  sa.row_bytes = ws_row_bytes(p->lmax, p->nnorth);
  sa.ring_i0 = p->d_ring_i0;
  sa.WS = WS;
  sa.EB = EB;
  sa.err = p->d_err;
  k_slice_phase<<<dim3(wv[1] - wv[0], 4 * sa.ngroups), kSliceThreads, 0, s>>>(sa);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

// ------------------------------------------------------------------ host side
namespace {
constexpr size_t kLbufCap = 2ull << 30;     // lambda-digit staging per wave

int eag_of(int lmax) {
  const double b = std::sqrt((2.0 * lmax + 1.0) / (4.0 * M_PI)) * (1.0 + 0x1p-30);
  return std::ilogb(b) + 1;
}
}

int fsht_split_tables_init(fsht_plan* p) {
  const int lmax = p->lmax;
  const size_t ntab = (size_t)tri_off(lmax + 1, lmax);
  FSHT_CUDA_TRY(cudaMalloc(&p->d_lamtab, sizeof(FshtLamRow) * (ntab ? ntab : 1)));
  FSHT_CUDA_TRY(cudaMalloc(&p->d_lam_off, sizeof(long long) * (lmax + 2)));
  FSHT_CUDA_TRY(cudaMalloc(&p->d_lam_offT, sizeof(long long) * (lmax + 2)));
  k_lam_table<<<(lmax + 1 + 127) / 128, 128, 0, p->stream>>>(lmax, p->d_lamtab);
  FSHT_LAUNCH_CHECK();
  // per q (pair order): 16 KB units of m(q)'s analysis tiles (l-rows) and synthesis tiles
  // (ring rows)
  std::vector<long long> off(lmax + 2, 0), offT(lmax + 2, 0);
  std::vector<int> ntl(lmax + 1), nkm(lmax + 1), nrb(lmax + 1), nkl(lmax + 1);
  for (int q = 0; q <= lmax; ++q) {
    const int m = (q & 1) ? lmax - (q >> 1) : (q >> 1);
    const int K = p->nnorth - p->h_ring_i0[m];
    ntl[q] = (lmax - m + 1 + 2 * kRows - 1) / (2 * kRows);
    nkm[q] = K > 0 ? (K + kKStep - 1) / kKStep : 0;
    nrb[q] = K > 0 ? (K + kSCRings - 1) / kSCRings : 0;
    nkl[q] = ((lmax - m) / 2 + 1 + kKStep - 1) / kKStep;
    off[q + 1] = off[q] + 2LL * ntl[q] * nkm[q];
    offT[q + 1] = offT[q] + 2LL * nrb[q] * nkl[q];
  }
  const size_t unit = (size_t)kSlices * kATileBytes;
  const size_t cap_units = kLbufCap / unit;
  // spin-2 plans stage lambda1 and lambda2: twice the analysis tiles
  const long long fa = p->pol ? 2 : 1;
  auto span = [&](int q0, int q1) -> size_t {
    return (size_t)std::max(fa * (off[q1] - off[q0]), fa * (offT[q1] - offT[q0]));
  };
  // waves: consecutive q ranges whose tiles (either layout) fit the staging buffer
  std::vector<int> waves;
  size_t lbuf_units = 0;
  for (int q0 = 0; q0 <= lmax;) {
    int q1 = q0 + 1;
    while (q1 <= lmax && span(q0, q1 + 1) <= cap_units) ++q1;
    int wv[kWaveInts] = {q0, q1, 0, 0, 0, 0, 0};
    for (int q = q0; q < q1; ++q) {
      wv[2] = std::max(wv[2], ntl[q]);
      wv[3] = std::max(wv[3], (nkm[q] * kKStep + kKChunk - 1) / kKChunk);
      wv[4] = std::max(wv[4], nrb[q]);
      wv[5] = std::max(wv[5], nkl[q]);
      wv[6] = std::max(wv[6], (nkl[q] * kKStep + kKChunk - 1) / kKChunk);
    }
    waves.insert(waves.end(), wv, wv + kWaveInts);
    lbuf_units = std::max(lbuf_units, span(q0, q1));
    p->wave_qmax = std::max(p->wave_qmax, q1 - q0);
    q0 = q1;
  }
  p->nwaves = (int)waves.size() / kWaveInts;
  p->h_waves = new (std::nothrow) int[waves.size()];
  if (!p->h_waves) {
    fsht_set_error("host allocation failed");
    return FSHT_ENOMEM;
  }
  std::copy(waves.begin(), waves.end(), p->h_waves);
  p->lbuf_bytes = std::max<size_t>(lbuf_units * unit, 256);
  FSHT_CUDA_TRY(cudaMemcpyAsync(p->d_lam_off, off.data(), sizeof(long long) * (lmax + 2),
                                cudaMemcpyHostToDevice, p->stream));
  FSHT_CUDA_TRY(cudaMemcpyAsync(p->d_lam_offT, offT.data(), sizeof(long long) * (lmax + 2),
                                cudaMemcpyHostToDevice, p->stream));
  FSHT_CUDA_TRY(cudaStreamSynchronize(p->stream));   // the offsets are stack vectors
  return FSHT_OK;
}

void fsht_split_wave_range(const fsht_plan* p, int w, int* q0, int* q1) {
  const int* wv = p->h_waves + kWaveInts * w;
  *q0 = wv[0];
  *q1 = wv[1];
}

int fsht_launch_split_lambda(fsht_plan* p, int w, unsigned char* lbuf, cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  LamArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.q0 = wv[0];
  a.cth = p->d_cth;
  a.sth = p->d_sth;
  a.pref = p->d_pref;
  a.ring_i0 = p->d_ring_i0;
  a.tab = p->d_lamtab;
  a.lam_off = p->d_lam_off;
  a.lbuf = lbuf;
  a.err = p->d_err;
  if (wv[4] == 0) return FSHT_OK;
  k_lambda_digits<<<dim3(wv[1] - wv[0], wv[4]), 128, 0, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

int fsht_launch_split_gemm(fsht_plan* p, int w, const unsigned char* WS, const int* EB,
                           const unsigned char* lbuf, double* alm, int nmaps_total, int k0,
                           int kc, int accumulate, cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  if (wv[3] == 0) return FSHT_OK;
  GemmArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  a.row_bytes = ws_row_bytes(p->lmax, p->nnorth);
  a.accumulate = accumulate;
  a.q0 = wv[0];
  a.ntmax = wv[2];
  a.ring_i0 = p->d_ring_i0;
  a.lam_off = p->d_lam_off;
  a.tab = p->d_lamtab;
  a.lbuf = lbuf;
  a.WS = WS;
  a.EB = EB;
  a.alm = alm;
  a.ld = nmaps_total;
  a.k0 = k0;
  a.kc = kc;
  a.pa = p->pa;
  a.err = p->d_err;
  a.part_steps = (p->split_part > 0 && p->split_part < kPartSteps) ? p->split_part : kPartSteps;
  a.nunits = a.ngroups * 2 * a.ntmax * (wv[1] - wv[0]);
  const size_t sm = kSmemG;
  FSHT_TRY(fsht_smem_limit((const void*)k_split_gemm, (size_t)(sm)));
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  // persistent: one CTA per SM, or fewer while another kernel needs SMs beside it
  const int cap = (p->gemm_ctas > 0 && p->gemm_ctas < nsm) ? p->gemm_ctas : nsm;
  const int grid = a.nunits < cap ? a.nunits : cap;
  if (grid > 0) k_split_gemm<<<grid, kThreadsG, sm, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

int fsht_launch_split_slice_alm(fsht_plan* p, int w, const double* alm, unsigned char* WS,
                                int* EB, int nmaps_total, int k0, int kc, cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  SliceAArgs a;
  a.alm = alm;
  a.ld = nmaps_total;
  a.k0 = k0;
  a.kc = kc;
  a.lmax = p->lmax;
  a.ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  a.q0 = wv[0];
  a.row_bytes = ws_row_bytes(p->lmax, p->nnorth);
  a.WS = WS;
  a.EB = EB;
  a.err = p->d_err;
  k_slice_alm<<<dim3(wv[1] - wv[0], 2, a.ngroups), 128, 0, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

int fsht_launch_split_lambdaT(fsht_plan* p, int w, unsigned char* lbuf, cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  if (wv[4] == 0) return FSHT_OK;
  LamTArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.q0 = wv[0];
  a.eag = eag_of(p->lmax);
  a.cth = p->d_cth;
  a.sth = p->d_sth;
  a.pref = p->d_pref;
  a.ring_i0 = p->d_ring_i0;
  a.tab = p->d_lamtab;
  a.lam_offT = p->d_lam_offT;
  a.lbuf = lbuf;
  a.err = p->d_err;
  k_lambda_digits_T<<<dim3(wv[1] - wv[0], wv[4]), 128, 0, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

int fsht_launch_split_synth(fsht_plan* p, int w, const unsigned char* WS, const int* EB,
                            const unsigned char* lbuf, double2* W, int kc, cudaStream_t s) {
  const int* wv = p->h_waves + kWaveInts * w;
  if (wv[4] == 0 || wv[6] == 0) return FSHT_OK;
  SynthArgs a;
  a.lmax = p->lmax;
  a.nnorth = p->nnorth;
  a.ngroups = (kc + kGroupMaps - 1) / kGroupMaps;
  a.row_bytes = ws_row_bytes(p->lmax, p->nnorth);
  a.q0 = wv[0];
  a.nrbmax = wv[4];
  a.eag = eag_of(p->lmax);
  a.nunits = a.ngroups * a.nrbmax * (wv[1] - wv[0]);
  a.ring_i0 = p->d_ring_i0;
  a.lam_offT = p->d_lam_offT;
  a.lbuf = lbuf;
  a.WS = WS;
  a.EB = EB;
  a.W = reinterpret_cast<double*>(W);
  a.kc = kc;
  a.err = p->d_err;
  const size_t sm = (size_t)kStagesS * kStageBytesS;
  FSHT_TRY(fsht_smem_limit((const void*)k_split_synth, (size_t)(sm)));
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int grid = a.nunits < nsm ? a.nunits : nsm;
  if (grid > 0) k_split_synth<<<grid, kThreadsG, sm, s>>>(a);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}
