// alm layout conversion between the square-real packing and healpy's m-major
// triangle (reference convert_alm_healpy1 / convert_alm_healpy_inv1,
// src/convert_alm.f90:34-56, 87-107; used by SHT.convert_alm_healpy, SHT.py:204-210).
//
// square : alm[c][l][k], Re a_lm at c = m (l >= m), Im a_lm at c = lmax+1-m, row l-m
// healpy : out[k][idx] complex (re, im), idx = m (2 lmax + 1 - m) / 2 + l
// A 32 (idx) x 32 (maps) tile is staged in shared memory so that both the reads
// (map index fastest) and the writes (idx fastest) are coalesced.
#include "common.cuh"

namespace {

// Order m's entries start at idx = m(2 lmax + 1 - m)/2 + m = m(2 lmax + 3 - m)/2.
__device__ __forceinline__ long long hp_start(int m, int lmax) {
  return (long long)m * (2 * lmax + 3 - m) / 2;
}
__device__ __forceinline__ void idx_to_lm(long long idx, int lmax, int& l, int& m) {
  // largest m with hp_start(m) <= idx: solve the quadratic, then fix rounding
  const double b = 2.0 * lmax + 3.0;
  const double disc = b * b - 8.0 * (double)idx;
  int mm = (int)floor((b - sqrt(disc > 0.0 ? disc : 0.0)) / 2.0);
  if (mm < 0) mm = 0;
  if (mm > lmax) mm = lmax;
  while (mm > 0 && hp_start(mm, lmax) > idx) --mm;
  while (mm < lmax && hp_start(mm + 1, lmax) <= idx) ++mm;
  m = mm;
  l = (int)(idx - (long long)mm * (2 * lmax + 1 - mm) / 2);
}

__global__ void k_square_to_healpy(const double* __restrict__ alm, double2* __restrict__ out,
                                   int lmax, int nmaps, long long nalm) {
  __shared__ double2 tile[32][33];
  const long long idx0 = (long long)blockIdx.x * 32;
  const int k0 = blockIdx.y * 32;
  const long long L1 = lmax + 1;
  const int tx = threadIdx.x, ty = threadIdx.y;   // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const long long idx = idx0 + r;
    const int k = k0 + tx;
    double2 v = make_double2(0.0, 0.0);
    if (idx < nalm && k < nmaps) {
      int l, m;
      idx_to_lm(idx, lmax, l, m);
      v.x = alm[((long long)m * L1 + l) * nmaps + k];
      if (m > 0) v.y = alm[((L1 - m) * L1 + (l - m)) * nmaps + k];
    }
    tile[r][tx] = v;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int k = k0 + r;
    const long long idx = idx0 + tx;
    if (idx < nalm && k < nmaps) out[(long long)k * nalm + idx] = tile[tx][r];
  }
}

__global__ void k_healpy_to_square(const double2* __restrict__ in, double* __restrict__ alm,
                                   int lmax, int nmaps, long long nalm) {
  __shared__ double2 tile[32][33];
  const long long idx0 = (long long)blockIdx.x * 32;
  const int k0 = blockIdx.y * 32;
  const long long L1 = lmax + 1;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < 32; r += 8) {
    const int k = k0 + r;
    const long long idx = idx0 + tx;
    if (idx < nalm && k < nmaps) tile[tx][r] = in[(long long)k * nalm + idx];
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const long long idx = idx0 + r;
    const int k = k0 + tx;
    if (idx < nalm && k < nmaps) {
      int l, m;
      idx_to_lm(idx, lmax, l, m);
      const double2 v = tile[r][tx];
      alm[((long long)m * L1 + l) * nmaps + k] = v.x;
      if (m > 0) alm[((L1 - m) * L1 + (l - m)) * nmaps + k] = v.y;
    }
  }
}

}  // namespace

extern "C" int fsht_convert_alm_healpy(fsht_plan* p, const double* alm, double* alm_hp, int nmaps) {
  if (!p || !alm || !alm_hp || nmaps < 1) {
    fsht_set_error("convert_alm_healpy: bad arguments");
    return FSHT_EINVAL;
  }
  const long long nalm = (long long)(p->lmax + 1) * (p->lmax + 2) / 2;
  dim3 grid((unsigned)((nalm + 31) / 32), (nmaps + 31) / 32);
  k_square_to_healpy<<<grid, dim3(32, 8), 0, p->stream>>>(alm, (double2*)alm_hp, p->lmax, nmaps,
                                                          nalm);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

extern "C" int fsht_convert_alm_healpy_inv(fsht_plan* p, const double* alm_hp, double* alm,
                                           int nmaps) {
  if (!p || !alm || !alm_hp || nmaps < 1) {
    fsht_set_error("convert_alm_healpy_inv: bad arguments");
    return FSHT_EINVAL;
  }
  const long long nalm = (long long)(p->lmax + 1) * (p->lmax + 2) / 2;
  dim3 grid((unsigned)((nalm + 31) / 32), (nmaps + 31) / 32);
  k_healpy_to_square<<<grid, dim3(32, 8), 0, p->stream>>>((const double2*)alm_hp, alm, p->lmax,
                                                          nmaps, nalm);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}
