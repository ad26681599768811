/*
 * ORACLE (test infrastructure): C restatement of the reference's per-m
 * associated-Legendre recursion, get_plm_recursive (src/get_plm_recursive.f90:17-136),
 * for the north rings i0..2 nside-1.  The NumPy oracle calls it through ctypes to
 * make the timed CPU baseline run at compiled speed; tests check it against the
 * NumPy restatement.
 *
 *   lambda_mm = pref (-sin theta)^m, pref = sqrt(diag_fac(m)/4/pi)
 *   lambda_l  = a_l cos(theta) lambda_{l-1} - b_l lambda_{l-2}
 *   a_l = sqrt(c3(l)/(c4(l)-m^2)), b_l = sqrt((c1(l)-m^2)/c2(l)) a_l
 * scaled = 0 seeds directly (the reference's nside <= 512 branch); scaled = 1
 * carries values as v * 2^(600 e) (e <= 0) and returns 0 while e < 0, replacing
 * the reference's nside > 512 "safe start" tables.
 * Spin 2 (pol = 1, get_plm_recursive.f90:101-125) also fills plm1 / plm2.
 * oracle_plm: outputs row-major (nr, lmax+1); columns < m are left untouched.
 * oracle_plm_sphere: the full-sphere table the reference's mat2alm/alm2mat use
 * (rows = kept rings i0..nring-1-i0, columns l = m..lmax), south ring i filled
 * from its mirror nring-1-i with sign (-1)^(l+m) (plm0, plm1) or (-1)^(l+m+1)
 * (plm2) (get_plm_recursive.f90:93-98, 128-134).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>

static void seed_scaled(double s, double pref, int m, double* cur, int* e) {
  int ex;
  double mt = frexp(s, &ex);
  double rm = 1.0, bm = mt;
  long long re = 0, be = ex;
  for (int k = m; k; k >>= 1) {
    if (k & 1) {
      int t;
      rm *= bm;
      re += be;
      rm = frexp(rm, &t);
      re += t;
    }
    if (k > 1) {
      int t;
      bm *= bm;
      be *= 2;
      bm = frexp(bm, &t);
      be += t;
    }
  }
  {
    int t;
    rm *= pref;
    rm = frexp(rm, &t);
    re += t;
  }
  if (m & 1) rm = -rm;
  *e = (re >= -300) ? 0 : (int)floor((double)(re + 300) / 600.0);
  *cur = ldexp(rm, (int)(re - 600LL * (*e)));
}

void oracle_plm(int m, int lmax, int nr, const double* cc, const double* ss, double pref,
                int scaled, int pol, double* plm0, double* plm1, double* plm2) {
  const int L = lmax + 1;
  double* a = (double*)__builtin_alloca(sizeof(double) * L);
  double* b = (double*)__builtin_alloca(sizeof(double) * L);
  double* lf = (double*)__builtin_alloca(sizeof(double) * L);
  double* nl = (double*)__builtin_alloca(sizeof(double) * L);
  for (int l = m + 1; l <= lmax; ++l) {
    const double c1 = (double)(l - 1) * (l - 1), c2 = (double)(2 * l - 3) * (2 * l - 1);
    const double c3 = (double)(2 * l - 1) * (2 * l + 1), c4 = (double)l * l;
    a[l] = sqrt(c3 / (c4 - (double)m * m));
    b[l] = sqrt((c1 - (double)m * m) / c2) * a[l];
  }
  if (pol) {
    const int m1 = m > 1 ? m : 1;
    for (int l = 0; l <= lmax; ++l) {
      lf[l] = (l <= m1) ? 0.0
                        : 2.0 * sqrt((double)(2 * l + 1) / (2 * l - 1) *
                                     (double)((long long)l * l - (long long)m * m));
      nl[l] = (l < 2) ? 0.0 : 1.0 / sqrt((double)(l + 2) * (l + 1) * (double)l * (l - 1));
    }
  }
#pragma omp parallel for schedule(static)
  for (int r = 0; r < nr; ++r) {
    const double c = cc[r], s = ss[r];
    double* out = plm0 + (size_t)r * L;
    double cur, prev = 0.0;
    int e = 0;
    if (scaled) {
      seed_scaled(s, pref, m, &cur, &e);
    } else {
      cur = pref * pow(-s, m);
    }
    out[m] = (e == 0) ? cur : 0.0;
    for (int l = m + 1; l <= lmax; ++l) {
      const double nx = a[l] * c * cur - b[l] * prev;
      prev = cur;
      cur = nx;
      if (e < 0 && fabs(cur) > 0x1p300) {
        cur *= 0x1p-600;
        prev *= 0x1p-600;
        ++e;
      }
      out[l] = (e == 0) ? cur : 0.0;
    }
    if (pol) {
      const double s2 = s * s, b_w = c / s2, two_on_s2 = 2.0 / s2, c_w = (double)m / s2;
      double* o1 = plm1 + (size_t)r * L;
      double* o2 = plm2 + (size_t)r * L;
      const double nm = (double)(2LL * m * (1 - m)) * nl[m];
      o1[m] = nm * out[m] * (0.5 - 1.0 / s2);
      o2[m] = nm * out[m] * c / s2;
      for (int l = m + 1; l <= lmax; ++l) {
        o1[l] = (out[l - 1] * lf[l] * b_w -
                 out[l] * (two_on_s2 * (double)((long long)l - (long long)m * m) + l * (l - 1.0))) *
                nl[l];
        o2[l] = (out[l - 1] * lf[l] - out[l] * (2.0 * c * (l - 1.0))) * c_w * nl[l];
      }
    }
  }
}

void oracle_plm_sphere(int m, int lmax, int nside, int i0, const double* cc_all,
                       const double* ss_all, double pref, int scaled, int pol, double* out0,
                       double* out1, double* out2) {
  const int nn = 2 * nside;             /* north rings incl. equator */
  const int nr = nn - i0;               /* north rows i0..nn-1 */
  const int n = lmax + 1 - m;
  const int L = lmax + 1;
  const int rlen = 4 * nside - 1 - 2 * i0;
  double* t0 = (double*)malloc(sizeof(double) * (size_t)nr * L);
  double* t1 = pol ? (double*)malloc(sizeof(double) * (size_t)nr * L) : t0;
  double* t2 = pol ? (double*)malloc(sizeof(double) * (size_t)nr * L) : t0;
  oracle_plm(m, lmax, nr, cc_all + i0, ss_all + i0, pref, scaled, pol, t0, t1, t2);
#pragma omp parallel for schedule(static)
  for (int row = 0; row < rlen; ++row) {
    const int ring = i0 + row;
    const int src = ring < nn ? ring : (4 * nside - 2 - ring);   /* mirror */
    const int south = ring >= nn;
    const double* a = (pol ? t1 : t0) + (size_t)(src - i0) * L;
    const double* b = t2 + (size_t)(src - i0) * L;
    double* o = (pol ? out1 : out0) + (size_t)row * n;
    double* o2 = pol ? out2 + (size_t)row * n : NULL;
    for (int j = 0; j < n; ++j) {
      const int l = m + j;
      const double sg = (south && ((l + m) & 1)) ? -1.0 : 1.0;
      o[j] = sg * a[l];
      if (pol) o2[j] = (south ? -sg : sg) * b[l];
    }
  }
  free(t0);
  if (pol) {
    free(t1);
    free(t2);
  }
  (void)out0;
}

/*
 * fft2mat_fast (src/fft_mapping.f90:19-68) in the reference's memory order, for the timed
 * CPU baseline: the FFT bins b are (npix, nsim) with the map index fastest (the reference's
 * fft(1:nsim, i1:i2) after its transposing FFT), and for each kept ring r the pair of bins
 * (j[r], j[r] + 1) becomes one row of the FFT matrix:
 *   mat1[r][k] = b[j[r]][k] f1[r] + b[j[r]+1][k] f2[r],
 *   mat2[r][k] = b[j[r]][k] f3[r] + b[j[r]+1][k] f4[r].
 * OpenMP over rings, like the reference's parallel loop (fft_mapping.f90:41).
 */
void oracle_fft2mat(int nsim, int rlen, const double* b, const long long* j, const double* f1,
                    const double* f2, const double* f3, const double* f4, double* mat1,
                    double* mat2) {
#pragma omp parallel for schedule(static)
  for (int r = 0; r < rlen; ++r) {
    const double* x0 = b + (size_t)j[r] * nsim;
    const double* x1 = x0 + nsim;
    double* o1 = mat1 + (size_t)r * nsim;
    double* o2 = mat2 + (size_t)r * nsim;
    const double a1 = f1[r], a2 = f2[r], a3 = f3[r], a4 = f4[r];
    for (int k = 0; k < nsim; ++k) {
      o1[k] = x0[k] * a1 + x1[k] * a2;
      o2[k] = x0[k] * a3 + x1[k] * a4;
    }
  }
}
