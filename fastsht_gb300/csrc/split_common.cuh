// Constants and helpers shared by the split-precision kernels (legendre_split.cu,
// legendre_split_pol.cu): tile geometry, the recursion seed and coefficients, the
// pair order of m, the triangular (l, m) table index and the WS row size.
#pragma once
#include "common.cuh"
#include "df64.cuh"
#include "tcgen05.cuh"

#include <cmath>

namespace {

constexpr int kRows = 128;          // UMMA M: rows of one parity per l-tile
constexpr int kCols = 128;          // UMMA N: 64 maps x {Re, Im}
constexpr int kGroupMaps = 64;
constexpr int kKStep = 16;          // rings per UMMA
constexpr int kSCRings = 128;       // rings per lambda-digit block
constexpr int kKChunk = 1024;       // rings per CTA (keeps levels 0 and 1 exact)
constexpr int kSlices = 4;
constexpr uint32_t kATileBytes = kRows * kKStep * 2;    // 4 KB per (k-step, digit)
constexpr uint32_t kBTileBytes = kCols * kKStep * 2;    // 4 KB per (k-step, digit)
// Synthesis B tiles carry three more digit planes, d1..d3 times 2^-8 (exact in BF16), so
// the level-4 products fold into the level-3 accumulator.
constexpr int kSynthPlanes = 7;
constexpr uint32_t kSynthBBytes = kSynthPlanes * kBTileBytes;   // 28 KB per l-step
constexpr int kThreads = 192;
// persistent analysis contractions: eight epilogue warps (two per TMEM lane quarter, one per
// half of the columns), then the copy thread's warp and the UMMA thread's warp
constexpr int kEpiThreads = 256;
constexpr int kThreadsG = kEpiThreads + 64;
constexpr int kEmptyExp = -4000;    // column exponent of an all-zero column
// Epilogue staging of the analysis GEMMs: each epilogue warp turns a 32-row x 16-column block
// of results around in shared memory, so that its global stores and reductions go out as
// 128-byte row segments (two rows per instruction) instead of 32 scattered 8-byte values.
// Column j of row r sits at j ^ (r & 15): both the row-wise writes and the column-wise reads
// of a warp touch each bank pair at most twice.
constexpr int kStgWarpDoubles = 32 * 16;
constexpr size_t kStgBytes = (size_t)(kEpiThreads / 32) * kStgWarpDoubles * sizeof(double);
__device__ __forceinline__ int stg_at(int r, int c) { return r * 16 + (c ^ (r & 15)); }

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

__device__ __forceinline__ int m_of_q(int q, int lmax) {
  return (q & 1) ? lmax - (q >> 1) : (q >> 1);
}
__host__ __device__ __forceinline__ long long tri_off(int m, int lmax) {
  return (long long)m * (2LL * lmax + 3 - m) / 2;
}

// per wave: q0, q1, max l-tiles, max ring K-chunks (analysis), max 128-ring blocks,
// max l-steps, max l K-chunks (synthesis)
constexpr int kWaveInts = 7;

// WS bytes per (m, parity, group): the analysis P tiles (rings) or the synthesis alm tiles
// (l of one parity), whichever is larger
size_t ws_row_bytes(int lmax, int nnorth) {
  const size_t nks = (size_t)(nnorth + kKStep - 1) / kKStep;
  const size_t nkl = (size_t)(lmax / 2 + 1 + kKStep - 1) / kKStep;
  const size_t a = nks * kSlices * kBTileBytes, b = nkl * kSynthBBytes;
  return a > b ? a : b;
}

// Levels 0..3 of one output element (FP32 accumulators, weights 1, 2^-8, 2^-16, 2^-24):
// levels 0 and 1 are exact integers, so their weighted sum is exact as an FP32 (hi, lo)
// pair (two-sum); levels 2 and 3 only touch lo.
__device__ __forceinline__ void combine_levels_pair(uint32_t v0, uint32_t v1, uint32_t v2,
                                                    uint32_t v3, float& hi, float& lo) {
  const float L0 = __uint_as_float(v0);
  const float L1f = __uint_as_float(v1) * 0x1p-8f;
  hi = L0 + L1f;
  const float bv = hi - L0;
  lo = ((L0 - (hi - bv)) + (L1f - bv)) +
       (__uint_as_float(v2) * 0x1p-16f + __uint_as_float(v3) * 0x1p-24f);
}

// The element times (fh + fl) 2^e as an FP64.  The product of the (hi, lo) pair with the
// df64 factor is formed on the FP32 pipe (the high product exact through fmaf, the cross
// terms in the low part, ~2^-46 relative), the power of two goes into the exponent fields
// and one FP64 addition joins the two parts: one FP64 instruction per element instead of
// five (two conversions, an addition, two multiplications).  Exponents below the FP64 range
// give 0, so an empty column (exponent kEmptyExp) writes zeros.
__device__ __forceinline__ double pair_scaled(float hi, float lo, float fh, float fl, int e) {
  const float p = __fmul_rn(hi, fh);
  float q = __fmaf_rn(hi, fh, -p);
  q = __fmaf_rn(hi, fl, q);
  q = __fmaf_rn(lo, fh, q);
  return dd_to_double(p, q, e);
}
__device__ __forceinline__ double levels_scaled(uint32_t v0, uint32_t v1, uint32_t v2,
                                                uint32_t v3, float fh, float fl, int e) {
  float hi, lo;
  combine_levels_pair(v0, v1, v2, v3, hi, lo);
  return pair_scaled(hi, lo, fh, fl, e);
}

// A positive or negative FP64 factor as a df64 pair (setup, once per row).
__device__ __forceinline__ void factor_pair(double x, float& fh, float& fl) {
  fh = __double2float_rn(x);
  fl = __double2float_rn(x - (double)fh);
}

}  // namespace
