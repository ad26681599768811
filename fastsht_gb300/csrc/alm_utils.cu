// alm utilities on the device, in the square-real alm layout [col][row][map] (map fastest):
// Re a_lm at col m, row l (row >= col); Im a_lm at col lmax+1-m, row l-m (row < col).
//
//   fsht_alm2cl    power / cross spectra   (reference alm2cl_TEB1 / alm2cl_T1,
//                                            src/alm2cl_TEB.f90:22-110)
//   fsht_alm_filter  alm *= win(l)          (filt_alm1, src/filt_alm.f90:16-37)
//   fsht_alm_norm    alm*fac(l) + shift(l), m = 0 scaled by m0 as well
//                                           (norm_alm1, src/norm_alm.f90:14-35)
//   fsht_cl2alm    Gaussian realisations with the 6 spectra TT EE BB TE TB EB
//                  (cl2alm_TEB1 / cl2alm_T1, src/cl2alm_TEB.f90:25-171)
//
// The reference draws its Gaussians from MKL's MCG31 stream, which is not available; these
// use a counter-based generator (SplitMix64 of (seed, field, position, map), Box-Muller), so
// realisations are reproducible per seed and independent of the launch shape, and the
// correlation step follows the reference's per-l factorisation.
#include "common.cuh"

#include <cmath>

namespace {

__device__ __forceinline__ void lm_of(int col, int row, int L1, int& l, int& m) {
  if (row >= col) {
    m = col;
    l = row;
  } else {
    m = L1 - col;
    l = row + m;
  }
}

// ------------------------------------------------------------------ alm2cl
// cl[l][k] = sum_m fac_m (a1_lm a2_lm)/(2l+1) over Re and Im parts, fac_0 = 1, fac_m = 2;
// l < lmin gives 0.  Thread per (l, map).
__global__ void k_alm2cl(const double* __restrict__ a1, const double* __restrict__ a2,
                         double* cl, int lmax, int nmaps, int lmin) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int l = blockIdx.y;
  if (k >= nmaps) return;
  const long long L1 = lmax + 1;
  double s = 0.0;
  if (l >= lmin) {
    for (int m = 0; m <= l; ++m) {
      const long long re = ((long long)m * L1 + l) * nmaps + k;
      double t = a1[re] * a2[re];
      if (m > 0) {
        const long long im = ((L1 - m) * L1 + (l - m)) * nmaps + k;
        t = 2.0 * (t + a1[im] * a2[im]);
      }
      s += t;
    }
    s /= (double)(2 * l + 1);
  }
  cl[(long long)l * nmaps + k] = s;
}

// ------------------------------------------------------------------ filter / norm
__global__ void k_alm_scale(const double* in, double* out, const double* __restrict__ fac,
                            const double* __restrict__ shift, double m0, int lmax, int nmaps) {
  const long long L1 = lmax + 1;
  const long long total = L1 * L1 * nmaps;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long pos = idx / nmaps;
    const int row = (int)(pos % L1), col = (int)(pos / L1);
    int l, m;
    lm_of(col, row, (int)L1, l, m);
    double v = in[idx] * fac[l];
    if (m == 0 && row >= col) v *= m0;
    out[idx] = shift ? v + shift[l] : v;
  }
}

// ------------------------------------------------------------------ cl2alm
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// N(0, 1) for (seed, field, position, map): two 53-bit uniforms, Box-Muller (cos branch).
__device__ __forceinline__ double gauss(unsigned long long seed, int field, long long pos, int k) {
  const unsigned long long c =
      splitmix64(seed ^ splitmix64(((unsigned long long)pos << 20) ^ ((unsigned long long)k << 2) ^
                                   (unsigned long long)field));
  const unsigned long long d = splitmix64(c);
  const double u1 = ((double)(c >> 11) + 0.5) * 0x1p-53;   // (0, 1)
  const double u2 = (double)(d >> 11) * 0x1p-53;           // [0, 1)
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

// Per l: a = sqrt(TT), b = TE/a, c = TB/a, u = sqrt(EE - b^2),
// v = (TT EB - TE TB)/(u TT), w = sqrt(BB - TB/TT/u^2 (EE TB - TE EB) - v EB / u);
// T = a g1, E = b g1 + u g2, B = c g1 + v g2 + w g3 with g ~ N(0, 1) at m = 0 and
// N(0, 1/2) per Re / Im part at m > 0; l < lmin gives 0.  ncl = 1: T only.
__global__ void k_cl2alm(const double* __restrict__ cl, int ncl, int lmin, int lmax, int nmaps,
                         unsigned long long seed, double* almT, double* almE, double* almB) {
  const long long L1 = lmax + 1;
  const long long total = L1 * L1 * nmaps;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long pos = idx / nmaps;
    const int k = (int)(idx % nmaps);
    const int row = (int)(pos % L1), col = (int)(pos / L1);
    int l, m;
    lm_of(col, row, (int)L1, l, m);
    if (l < lmin) {
      almT[idx] = 0.0;
      if (ncl == 6) {
        almE[idx] = 0.0;
        almB[idx] = 0.0;
      }
      continue;
    }
    const double sd = (m == 0) ? 1.0 : 0.70710678118654752440;
    const double g1 = sd * gauss(seed, 0, pos, k);
    if (ncl == 1) {
      almT[idx] = g1 * sqrt(cl[l]);
      continue;
    }
    const double g2 = sd * gauss(seed, 1, pos, k), g3 = sd * gauss(seed, 2, pos, k);
    const double tt = cl[l * 6 + 0], ee = cl[l * 6 + 1], bb = cl[l * 6 + 2];
    const double te = cl[l * 6 + 3], tb = cl[l * 6 + 4], eb = cl[l * 6 + 5];
    double a = 0, b = 0, c = 0, u = 0, v = 0, w = 0;
    if (tt > 0.0) {
      a = sqrt(tt);
      b = te / a;
      c = tb / a;
      const double u2 = ee - b * b;
      u = u2 > 0.0 ? sqrt(u2) : 0.0;
      if (u > 0.0) {
        v = (tt * eb - te * tb) / (u * tt);
        const double w2 = bb - tb / tt / (u * u) * (ee * tb - te * eb) - v * eb / u;
        w = w2 > 0.0 ? sqrt(w2) : 0.0;
      } else {
        w = bb > 0.0 ? sqrt(bb) : 0.0;
      }
    } else {   // no temperature power: E and B alone
      u = ee > 0.0 ? sqrt(ee) : 0.0;
      v = u > 0.0 ? eb / u : 0.0;
      const double w2 = bb - v * v;
      w = w2 > 0.0 ? sqrt(w2) : 0.0;
    }
    almT[idx] = a * g1;
    almE[idx] = b * g1 + u * g2;
    almB[idx] = c * g1 + v * g2 + w * g3;
  }
}

int grid_for(long long total) {
  long long g = (total + 255) / 256;
  return (int)(g > 152LL * 64 ? 152LL * 64 : (g < 1 ? 1 : g));
}

int check_sizes(int lmax, int nmaps) {
  if (lmax < 0 || nmaps < 1) {
    fsht_set_error("need lmax >= 0 and nmaps >= 1 (got %d, %d)", lmax, nmaps);
    return FSHT_EINVAL;
  }
  return FSHT_OK;
}

}  // namespace

extern "C" int fsht_alm2cl(const double* alm1, const double* alm2, double* cl, int lmax,
                           int nmaps, int lmin, void* stream) {
  FSHT_TRY(check_sizes(lmax, nmaps));
  if (!alm1 || !cl) {
    fsht_set_error("alm2cl: null pointer");
    return FSHT_EINVAL;
  }
  dim3 grid((nmaps + 127) / 128, lmax + 1);
  k_alm2cl<<<grid, 128, 0, (cudaStream_t)stream>>>(alm1, alm2 ? alm2 : alm1, cl, lmax, nmaps,
                                                   lmin < 0 ? 0 : lmin);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

extern "C" int fsht_alm_filter(double* alm, const double* win, int lmax, int nmaps, void* stream) {
  FSHT_TRY(check_sizes(lmax, nmaps));
  if (!alm || !win) {
    fsht_set_error("alm_filter: null pointer");
    return FSHT_EINVAL;
  }
  const long long total = (long long)(lmax + 1) * (lmax + 1) * nmaps;
  k_alm_scale<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(alm, alm, win, nullptr, 1.0,
                                                                  lmax, nmaps);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

extern "C" int fsht_alm_norm(const double* alm_in, double* alm_out, const double* fac,
                             const double* shift, double m0, int lmax, int nmaps, void* stream) {
  FSHT_TRY(check_sizes(lmax, nmaps));
  if (!alm_in || !alm_out || !fac || !shift) {
    fsht_set_error("alm_norm: null pointer");
    return FSHT_EINVAL;
  }
  const long long total = (long long)(lmax + 1) * (lmax + 1) * nmaps;
  k_alm_scale<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(alm_in, alm_out, fac, shift, m0,
                                                                  lmax, nmaps);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

extern "C" int fsht_cl2alm(const double* cl, int ncl, int lmin, int lmax, int nmaps,
                           unsigned long long seed, double* almT, double* almE, double* almB,
                           void* stream) {
  FSHT_TRY(check_sizes(lmax, nmaps));
  if (ncl != 1 && ncl != 6) {
    fsht_set_error("cl2alm: ncl = %d must be 1 (TT) or 6 (TT EE BB TE TB EB)", ncl);
    return FSHT_EINVAL;
  }
  if (!cl || !almT || (ncl == 6 && (!almE || !almB))) {
    fsht_set_error("cl2alm: null pointer");
    return FSHT_EINVAL;
  }
  const long long total = (long long)(lmax + 1) * (lmax + 1) * nmaps;
  k_cl2alm<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(cl, ncl, lmin < 0 ? 0 : lmin, lmax,
                                                               nmaps, seed, almT, almE, almB);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}
