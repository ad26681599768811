// Shared device/host helpers for the fastsht_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

#define FSHT_HD __host__ __device__ __forceinline__

// ---------------------------------------------------------------- complex FP64
FSHT_HD double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
FSHT_HD double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
FSHT_HD double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
FSHT_HD double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
FSHT_HD double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// ---------------------------------------------------------------- ring geometry
// Ring i of 4*nside-1: start pixel and length (reference get_ring_info,
// src/sht_data_init.f90:644-686).
FSHT_HD long long ring_start(int ns, int i) {
  long long n = ns;
  if (i < ns) return 2LL * i * (i + 1);
  if (i < 3 * ns - 1) return 2 * n + 4 * n * i - 2 * n * n;
  long long r = 4 * n - i;
  return 12 * n * n - 2 * (r - 1) * r;
}
FSHT_HD int ring_len(int ns, int i) {
  if (i < ns) return 4 * (i + 1);
  if (i < 3 * ns - 1) return 4 * ns;
  return 4 * (4 * ns - 1 - i);
}
// The first pixel of north ring i sits at phi0 = pi * s / n with s in {0, 1}:
// cap rings phi0 = pi/(4(i+1)) = pi/n; belt rings phi0 = pi/(4 nside) when
// (i+1-nside) is even, else 0 (HEALPix pix2ang, used by SHT.py:47-50).
FSHT_HD int ring_phase_flag(int ns, int i) {
  if (i < ns) return 1;
  return ((i + 1 - ns) % 2 == 0) ? 1 : 0;
}

// ---------------------------------------------------------------- plan
struct FshtRingFFT {
  int n;          // ring length
  int nd;         // DFT length: n (north + i south packed), or n/2 (each ring alone as its
                  // even/odd samples packed) when the packed transform exceeds shared memory
  int P;          // transform size: nd (power of two) or the Bluestein size 2^logT or 3*2^logT
  int logT;       // log2 of the power-of-two factor of P
  int r3;         // 1 when P = 3 * 2^logT
  int bluestein;  // 1 when nd is not a power of two
  long long chirp_off;  // offset (double2) of w_j = exp(-i pi j^2/nd), j < nd
  long long bhat_off;   // offset (double2) of the filter spectrum (transform order), P entries
  long long rtw_off;    // nd = n/2 only: offset of exp(-2 pi i k / n), k <= nd
};

// Transform size of a DFT of nd points: nd itself when nd is a power of two, else the
// smallest 2^k or 3*2^k >= 2 nd - 1 (Bluestein's linear convolution of length 2 nd - 1).
FSHT_HD void fsht_ring_fft_size(FshtRingFFT& r) {
  const int n = r.nd;
  r.r3 = 0;
  if ((n & (n - 1)) == 0) {
    r.bluestein = 0;
    r.P = n;
    int l = 0;
    while ((1 << l) < n) ++l;
    r.logT = l;
    return;
  }
  r.bluestein = 1;
  const int need = 2 * n - 1;
  int l2 = 0, l3 = 0;
  while ((1 << l2) < need) ++l2;
  while (3 * (1 << l3) < need) ++l3;
  if (3 * (1 << l3) < (1 << l2)) {
    r.P = 3 << l3;
    r.logT = l3;
    r.r3 = 1;
  } else {
    r.P = 1 << l2;
    r.logT = l2;
  }
}

// Twiddle table, packed per pass so that the threads of a warp read consecutive entries:
//   radix-4 part: for each span S = 2^s, s = 3..logTmax, at 3 (2^s - 8) / 4 the triples
//                 (w^j, w^2j, w^3j), w = exp(-2 pi i / S), j < S/4
//   radix-3 part: for each size P = 3 * 2^k, k = 0..log2(P3max / 3), at R4 + 2 (2^k - 1) the
//                 pairs (w^j, w^2j), w = exp(-2 pi i / P), j < 2^k
FSHT_HD long long fsht_tw_r4_entries(int Tmax) { return Tmax >= 8 ? 3LL * (2 * Tmax - 8) / 4 : 0; }
FSHT_HD long long fsht_tw_entries(int Tmax, int P3max) {
  return fsht_tw_r4_entries(Tmax) + (P3max > 0 ? 2LL * (2 * (P3max / 3) - 1) : 0);
}

// Split-precision form: per (l, m) row of the scaled recursion (legendre_split.cu).
struct FshtLamRow {
  double beta;   // mu_l = x mu_{l-1} - beta mu_{l-2}
  double dm;     // D_l = prod_{k=m+1..l} a_k = dm 2^dx, dm in [1, 2)
  int erow;      // EA(l) - dx: digit exponent of row l before the per-ring offset
  int dx;
};

// Spin-2 split form: per (l, m) factors of lambda1 / lambda2 (legendre_split_pol.cu).
struct FshtPolRow {
  double c1, c2, c3, c4;
};

struct fsht_plan {
  int nside, lmax, nring, nnorth;  // nnorth = 2*nside (north rings incl. equator)
  long long npix;
  int nmaps_max, kchunk;           // maps per workspace pass
  int pol, precision;
  cudaStream_t stream;
  double pa;                       // 4 pi / npix (sht_data_init.f90:18)
  // device tables
  double* d_cth;                   // cos(theta_i), i < 2 nside
  double* d_sth;                   // sin(theta_i)
  double* d_pref;                  // sqrt(diag_fac(m) / (4 pi)), m <= lmax
  int* d_ring_i0;                  // first kept ring for order m (m <= lmax)
  int* h_ring_i0;
  FshtRingFFT* d_rfft;             // per north ring
  double2* d_chirp;                // Bluestein chirps
  double2* d_rtw;                  // half-length rings: exp(-2 pi i k / n)
  double2* d_bhat;                 // Bluestein filter spectra
  double2* d_tw;                   // twiddles, packed per pass (fsht_tw_entries)
  long long fft_chirp_total, fft_bhat_total, fft_rtw_total;   // entries of the three tables
  // df64 copies (float4 = {re hi, im hi, re lo, im lo}) of the twiddle, chirp, filter and
  // half-ring tables: split-precision plans only (their forward FFT runs in df64)
  float4* d_tw_df;
  float4* d_chirp_df;
  float4* d_bhat_df;
  float4* d_rtw_df;
  float4* d_tw16_df;               // the df64 radix-16 passes' twiddles (fft_r16.cuh)
  int Pmax;                        // largest transform size (shared-memory sizing)
  int Tmax, logTmax, P3max;        // twiddle tables: largest power-of-two factor, largest 3*2^k size
  // workspace: phase matrices [m][i][k] x 2 complex, one per buffer
  double2* d_work;
  size_t work_bytes;
  int nbuf;
  size_t fft_smem;                 // dynamic smem of the ring FFT kernels (largest segment)
  // ring segments launched separately so rings with small transforms get 2 CTAs per SM:
  // {first ring, end ring, dynamic smem bytes} per segment
  int fft_nseg;
  long long fft_seg[3 * 8];
  int fft_seg_pmin[8];             // smallest transform size of each segment
  int fft_seg_gen[8];              // 1: the segment has Bluestein, radix-3 or half-length rings
  int fft_mpb, fft_threads;        // ring-FFT launch shape (0: heuristic), set by the autotuner
  // contraction tile shapes (0: defaults), set by the autotuner or fsht_plan_set_contraction:
  // FP64 analysis maps per CTA (32 | 64) and rings per chunk (spin 0: 8 | 16 | 32, spin 2:
  // 8 | 16); split GEMMs' ring-part length in k-steps of 16 rings (16 | 32 | 64)
  int ana_mt, ana_rc, split_part;
  struct FshtProfile* prof;        // non-null while per-kernel timing is on
  int* d_err;                      // device error word (bounded waits that expired)
  // split-precision form: sliced phase tiles and their column exponents, the scaled
  // recursion rows, and the lambda-digit staging buffer with its waves of m
  unsigned char* d_ws;
  int* d_eb;
  size_t ws_bytes;
  FshtLamRow* d_lamtab;            // triangular, (l, m) at m(2 lmax + 3 - m)/2 + l - m
  long long* d_lam_off;            // per pair-ordered index q: first 16 KB tile unit
  long long* d_lam_offT;           // the same for the synthesis (ring-row) tile layout
  int* h_waves;                    // per wave: see kWaveInts in legendre_split.cu
  int nwaves;
  unsigned char* d_lbuf;
  size_t lbuf_bytes;
  // plans that own their workspace: lambda-digit tiles one wave ahead on an auxiliary
  // stream, alternating between d_lbuf and d_lbuf2 (ev: fork, join, tiles ready x2,
  // contraction done x2); null / unused in table-only plans and their job views
  cudaStream_t aux;
  unsigned char* d_lbuf2;
  cudaEvent_t ev[6];
  // host-buffer entry points: copy stream and its events (fork, maps landed, wave done, join)
  cudaStream_t xfer;
  cudaEvent_t evx[4];
  // fsht_t2alm_host: 0 = maps that lie in one fsht_host_alloc block are read in place by the
  // forward FFT over the host link (no staging copy), 1 = maps are always copied first;
  // host_chunked: read in place in chunks, each chunk's contraction beside the next chunk's
  // reads (measured slower than one chunk on GB300; kept as an option)
  int host_staged, host_chunked;
  // spin-0 split analysis: slicing one wave ahead on a second auxiliary stream into the other
  // half of d_ws / d_eb (events: fork, join, slice done x2); null in job views
  cudaStream_t aux2;
  cudaEvent_t evs[4];
  // fsht_t2alm_host's chunked in-place route (split form): the contraction of a chunk of maps
  // on high-priority copies of the plan's streams while the next chunk's forward FFT reads the
  // host link on the plan's stream (events: fork, FFT done x2, contraction done x2); the GEMM's
  // persistent grid capped at gemm_ctas CTAs meanwhile (0 = one per SM)
  cudaStream_t hp_main, hp_aux, hp_aux2;
  cudaEvent_t evh[5];
  int gemm_ctas;
  int wave_qmax;                   // most orders in one wave
  FshtPolRow* d_poltab;            // spin-2 plans only, same triangular index as d_lamtab
};

// ---------------------------------------------------------------- status codes
#include "../../include/fastsht.h"

void fsht_set_error(const char* fmt, ...);
// Lets kernel `func` take at least `bytes` of dynamic shared memory on the current device.  The
// attribute is set only when the limit has to grow (once per kernel and device in practice):
// changing a function's attributes is not a launch-path operation and can wait for that
// function's launches in flight, which would tie the enqueueing thread to the GPU.
int fsht_smem_limit(const void* func, size_t bytes);

#define FSHT_CUDA_TRY(expr)                                                   \
  do {                                                                        \
    cudaError_t _e = (expr);                                                  \
    if (_e != cudaSuccess) {                                                  \
      fsht_set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr,              \
                     cudaGetErrorString(_e));                                 \
      return FSHT_ECUDA;                                                      \
    }                                                                         \
  } while (0)

#define FSHT_TRY(expr)       \
  do {                       \
    int _rc = (expr);        \
    if (_rc) return _rc;     \
  } while (0)

#define FSHT_LAUNCH_CHECK()                                                   \
  do {                                                                        \
    cudaError_t _e = cudaGetLastError();                                      \
    if (_e != cudaSuccess) {                                                  \
      fsht_set_error("%s:%d: kernel launch: %s", __FILE__, __LINE__,          \
                     cudaGetErrorString(_e));                                 \
      return FSHT_ECUDA;                                                      \
    }                                                                         \
  } while (0)

// ---------------------------------------------------------------- internal API
struct FshtFftLayout {
  int Pmax, Tmax, logTmax, P3max, nblue, nhalf;
  long long chirp_total, bhat_total, rtw_total;
  size_t smem;
};
// Host-side FFT table layout for nside/lmax; fills rfs[2 nside] and blue_rings
// (indices of Bluestein rings) when non-null.
int fsht_fft_layout(int nside, int lmax, FshtFftLayout* lay, FshtRingFFT* rfs, int* blue_rings);
// Fills the twiddle and Bluestein tables at p->d_tw / d_chirp / d_bhat (device
// ring descriptors at p->d_rfft must already be in place).  Allocates nothing.
int fsht_fft_tables_fill(fsht_plan* p, const int* d_blue_rings, int nblue, cudaStream_t s);
int fsht_fft_tables_init(fsht_plan* p);
int fsht_launch_ring_fft_fwd(fsht_plan* p, const double* maps, long long map_stride,
                             int kc, double2* W, cudaStream_t s);
// df64 tables of a split-precision plan (after fsht_fft_tables_init) and the df64 forward and
// inverse transforms, which fsht_launch_ring_fft_fwd / _inv select when they exist.
int fsht_fft_df_tables_init(fsht_plan* p);
int fsht_launch_ring_fft_fwd_df(fsht_plan* p, const double* maps, long long map_stride,
                                int kc, int k0, int kb, double2* W, cudaStream_t s);
// The forward transform of maps [k0, k0 + kb) of a chunk of kc maps (W keeps the chunk's
// map stride kc), for transfers that land in parts.
int fsht_launch_ring_fft_fwd_part(fsht_plan* p, const double* maps, long long map_stride,
                                  int kc, int k0, int kb, double2* W, cudaStream_t s);
// Pair-order range [q0, q1) of the orders in wave w of a split-precision plan.
void fsht_split_wave_range(const fsht_plan* p, int w, int* q0, int* q1);
int fsht_launch_ring_fft_inv_df(fsht_plan* p, const double2* W, double* maps,
                                long long map_stride, int kc, cudaStream_t s);
// Maps per CTA of the ring-FFT launches when the autotuner has not set one.
int fsht_fft_maps_per_block(int kc, int nrings);
int fsht_launch_ring_fft_inv(fsht_plan* p, const double2* W, double* maps,
                             long long map_stride, int kc, cudaStream_t s);
int fsht_launch_fourier_residual(fsht_plan* p, const double2* X, double2* GR, int kc,
                                 int prefix, cudaStream_t s);
int fsht_launch_ring_skip(fsht_plan* p, cudaStream_t s);
// Legendre contraction, FP64.  alm layout: [col][l][k] with ld = nmaps total,
// k offset k0.  which: bit0 = E (or T), bit1 = B.
int fsht_launch_analysis_fp64(fsht_plan* p, int spin, const double2* WQ,
                              const double2* WU, double* almE, double* almB,
                              int nmaps_total, int k0, int kc, int accumulate,
                              int which, cudaStream_t s);
// Split-precision form.  WS / EB: digit tiles and column exponents of one wave of m.
size_t fsht_split_ws_bytes(const fsht_plan* p, int kc);
size_t fsht_split_eb_bytes(const fsht_plan* p, int kc);
// Spin-0 analysis of one chunk (BF16 digits on tcgen05).  Tables (plan creation): recursion
// rows, per-m tile offsets, waves of m and the staging size.  Per wave w: slice cuts the
// {S, D} matrix W of the wave's orders into digit tiles WS and column exponents EB, lambda
// writes the wave's lambda digit tiles into lbuf, gemm contracts them into alm (stores, or
// adds when accumulate).
int fsht_split_tables_init(fsht_plan* p);
int fsht_launch_split_slice(fsht_plan* p, int w, const double2* W, unsigned char* WS, int* EB,
                            int kc, cudaStream_t s);
int fsht_launch_split_lambda(fsht_plan* p, int w, unsigned char* lbuf, cudaStream_t s);
int fsht_launch_split_gemm(fsht_plan* p, int w, const unsigned char* WS, const int* EB,
                           const unsigned char* lbuf, double* alm, int nmaps_total, int k0,
                           int kc, int accumulate, cudaStream_t s);
// Split-precision synthesis of one chunk into W = {G_N, G_S}: per wave, slice_alm cuts alm
// into digit tiles WS / exponents EB, lambdaT writes ring-row lambda tiles, synth contracts
// them.
int fsht_launch_split_slice_alm(fsht_plan* p, int w, const double* alm, unsigned char* WS,
                                int* EB, int nmaps_total, int k0, int kc, cudaStream_t s);
int fsht_launch_split_lambdaT(fsht_plan* p, int w, unsigned char* lbuf, cudaStream_t s);
// Split-precision spin-2 analysis: lambda1/lambda2 digit tiles per wave, then the E/B
// contraction (which: bit0 E, bit1 B) against the Q and U digit tiles of k_slice_phase.
int fsht_split_pol_tables_init(fsht_plan* p);
// Split-precision spin-2 synthesis (E/B -> {G_N, G_S} of Q and U) per wave: lambda1/lambda2
// ring-row tiles, then the four-pass contraction against the E and B alm tiles.
int fsht_launch_split_lambdaT_pol(fsht_plan* p, int w, unsigned char* lbuf, cudaStream_t s);
int fsht_launch_split_synth_pol(fsht_plan* p, int w, const unsigned char* WSE, const int* EBE,
                                const unsigned char* WSB, const int* EBB,
                                const unsigned char* lbuf, double2* WQ, double2* WU, int kc,
                                cudaStream_t s);
int fsht_launch_split_lambda_pol(fsht_plan* p, int w, unsigned char* lbuf, cudaStream_t s);
int fsht_launch_split_gemm_pol(fsht_plan* p, int w, const unsigned char* WSQ, const int* EBQ,
                               const unsigned char* WSU, const int* EBU,
                               const unsigned char* lbuf, double* almE, double* almB,
                               int nmaps_total, int k0, int kc, int accumulate, int which,
                               cudaStream_t s);
int fsht_launch_split_synth(fsht_plan* p, int w, const unsigned char* WS, const int* EB,
                            const unsigned char* lbuf, double2* W, int kc, cudaStream_t s);
int fsht_launch_synthesis_fp64(fsht_plan* p, int spin, const double* almE,
                               const double* almB, double2* WQ, double2* WU,
                               int nmaps_total, int k0, int kc, cudaStream_t s);
