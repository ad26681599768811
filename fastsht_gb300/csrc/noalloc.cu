// Allocation-free temperature analysis (fsht_t2alm_noalloc).
//
// Some callers cannot allocate device memory at the point where they want a
// transform: a host application that reserved the whole GPU for its own memory
// pool at start-up and hands its plug-ins device buffers but no right to call
// cudaMalloc, or a latency-critical loop where cudaMalloc/cudaFree would
// synchronise the device and stall other streams.  For them this entry point runs
// map -> alm without a plan and without any allocation: the ring-FFT tables, the
// recursion seeds and the phase-matrix scratch all live in one fixed array of
// device memory that is part of the library image (kNoAllocScratchBytes, held by
// every GPU that loads the library until the process exits).  The caller passes
// only the input maps and the output alm.
//
// The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call before
// any stream capture.  All calls share the array, so calls whose work overlaps on
// the GPU (different streams, or different host threads) race with each other;
// calls on one stream are ordered and safe.  Every byte a call reads from the
// array is written earlier in the same call, so nothing needs clearing between
// calls.
#include "common.cuh"

#include <cmath>
#include <mutex>

namespace {

// 32 MiB: enough for every nside <= 256 at any lmax <= 4 nside (nside 256 at lmax 1024
// runs one map per pass, about 6.7 MiB of tables plus 16 MiB of phase matrix), for many
// maps per pass below that, and for nside 512 up to lmax 167 (the FFT tables alone take
// about 26.7 MiB there).  Every other size is rejected with FSHT_EUNSUPPORTED.
constexpr size_t kNoAllocScratchBytes = 32ull << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct ScratchLayout {
  size_t cth, sth, pref, ring_i0, rfs, blue, tw, chirp, bhat, work, end;
};

ScratchLayout layout_for(int nside, int lmax, const FshtFftLayout& f) {
  const int nn = 2 * nside;
  ScratchLayout L;
  size_t o = 0;
  L.cth = o;     o = align256(o + sizeof(double) * nn);
  L.sth = o;     o = align256(o + sizeof(double) * nn);
  L.pref = o;    o = align256(o + sizeof(double) * (lmax + 1));
  L.ring_i0 = o; o = align256(o + sizeof(int) * (lmax + 1));
  L.rfs = o;     o = align256(o + sizeof(FshtRingFFT) * nn);
  L.blue = o;    o = align256(o + sizeof(int) * nn);
  L.tw = o;      o = align256(o + sizeof(double2) * (size_t)(fsht_tw_entries(f.Tmax, f.P3max) + 1));
  L.chirp = o;   o = align256(o + sizeof(double2) * (size_t)(f.chirp_total > 0 ? f.chirp_total : 1));
  L.bhat = o;    o = align256(o + sizeof(double2) * (size_t)(f.bhat_total > 0 ? f.bhat_total : 1));
  L.work = o;
  L.end = o;
  return L;
}

// Ring geometry, recursion seeds and FFT ring descriptors, written into the
// scratch by one block.  Same formulas as plan creation (HEALPix pix2loc for
// theta, diag_fac product for the seed prefactor); every ring is kept for every
// m (no ring skip: the skipped terms are below 1e-20 relative).
__global__ void k_noalloc_tables(int nside, int lmax, double* cth, double* sth, double* pref,
                                 int* ring_i0, FshtRingFFT* rfs, int* blue) {
  const int nn = 2 * nside;
  const double npix = 12.0 * nside * nside;
  const double fact2 = 4.0 / npix;
  const double fact1 = (double)(2 * nside) * fact2;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) {
    const int ir = i + 1;
    double th;
    if (ir < nside) {
      const double tmp = (double)ir * (double)ir * fact2;
      const double z = 1.0 - tmp;
      th = (z > 0.99) ? atan2(sqrt(tmp * (2.0 - tmp)), z) : acos(z);
    } else {
      th = acos((double)(2 * nside - ir) * fact1);
    }
    cth[i] = cos(th);
    sth[i] = sin(th);
  }
  for (int m = threadIdx.x; m <= lmax; m += blockDim.x) ring_i0[m] = 0;
  if (threadIdx.x == 0) {
    double df = 1.0;
    for (int m = 0; m <= lmax; ++m) {
      if (m > 0) df = df * (2 * m + 1) / 2 / m;
      pref[m] = sqrt(df / 4 / M_PI);
    }
    long long chirp_total = 0, bhat_total = 0;
    int nblue = 0;
    for (int i = 0; i < nn; ++i) {
      FshtRingFFT r;
      r.n = ring_len(nside, i);
      r.nd = r.n;
      r.rtw_off = 0;
      fsht_ring_fft_size(r);
      r.chirp_off = 0;
      r.bhat_off = 0;
      if (r.bluestein) {
        r.chirp_off = chirp_total;
        r.bhat_off = bhat_total;
        chirp_total += r.n;
        bhat_total += r.P;
        blue[nblue++] = i;
      }
      rfs[i] = r;
    }
  }
}

int scratch_address(void** out) {
  int dev = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    fsht_set_error("t2alm_noalloc: device ordinal %d above %d", dev, kMaxDevices - 1);
    return FSHT_EUNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      fsht_set_error("t2alm_noalloc: cudaGetSymbolAddress of the static scratch failed: %s",
                     cudaGetErrorString(e));
      return FSHT_ECUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return FSHT_OK;
}

}  // namespace

extern "C" int fsht_t2alm_noalloc(int nside, int lmax, const double* maps, double* alm,
                                  int nmaps, void* stream) {
  if (nside < 1 || (nside & (nside - 1)) || nside > 2048) {
    fsht_set_error("t2alm_noalloc: nside = %d must be a power of two in [1, 2048]", nside);
    return FSHT_EINVAL;
  }
  if (lmax < 0 || lmax > 4 * nside) {
    fsht_set_error("t2alm_noalloc: lmax = %d outside [0, 4*nside]", lmax);
    return FSHT_EINVAL;
  }
  if (nmaps < 1 || !maps || !alm) {
    fsht_set_error("t2alm_noalloc: need nmaps >= 1 and non-null maps/alm");
    return FSHT_EINVAL;
  }
  FshtFftLayout f;
  int rc = fsht_fft_layout(nside, lmax, &f, nullptr, nullptr);
  if (rc) return rc;
  if (f.nhalf > 0) {
    fsht_set_error("t2alm_noalloc: nside %d needs half-length ring transforms; use fsht_t2alm",
                   nside);
    return FSHT_EUNSUPPORTED;
  }
  const ScratchLayout L = layout_for(nside, lmax, f);
  const size_t per_map = (size_t)(lmax + 1) * 2 * nside * 2 * sizeof(double2);
  if (L.work + per_map > kNoAllocScratchBytes) {
    fsht_set_error("t2alm_noalloc: nside %d / lmax %d needs %zu bytes of scratch for one map, "
                   "above the %zu-byte static scratch; use fsht_t2alm with a plan", nside, lmax,
                   L.work + per_map, kNoAllocScratchBytes);
    return FSHT_EUNSUPPORTED;
  }
  void* base_v = nullptr;
  if ((rc = scratch_address(&base_v))) return rc;
  unsigned char* base = static_cast<unsigned char*>(base_v);
  const int kc_max = (int)((kNoAllocScratchBytes - L.work) / per_map);

  // A plan-shaped view of the scratch; nothing in it owns memory.
  fsht_plan p;
  memset(&p, 0, sizeof(p));
  p.nside = nside;
  p.lmax = lmax;
  p.nring = 4 * nside - 1;
  p.nnorth = 2 * nside;
  p.npix = 12LL * nside * nside;
  p.nmaps_max = nmaps;
  p.kchunk = kc_max < nmaps ? kc_max : nmaps;
  p.stream = (cudaStream_t)stream;
  p.pa = 4.0 * M_PI / (double)p.npix;
  p.d_cth = reinterpret_cast<double*>(base + L.cth);
  p.d_sth = reinterpret_cast<double*>(base + L.sth);
  p.d_pref = reinterpret_cast<double*>(base + L.pref);
  p.d_ring_i0 = reinterpret_cast<int*>(base + L.ring_i0);
  p.d_rfft = reinterpret_cast<FshtRingFFT*>(base + L.rfs);
  p.d_tw = reinterpret_cast<double2*>(base + L.tw);
  p.d_chirp = reinterpret_cast<double2*>(base + L.chirp);
  p.d_bhat = reinterpret_cast<double2*>(base + L.bhat);
  p.d_work = reinterpret_cast<double2*>(base + L.work);
  p.Pmax = f.Pmax;
  p.Tmax = f.Tmax;
  p.logTmax = f.logTmax;
  p.P3max = f.P3max;
  p.fft_smem = f.smem;
  p.fft_nseg = 1;
  p.fft_seg[0] = 0;
  p.fft_seg[1] = 2 * nside;
  p.fft_seg[2] = (long long)f.smem;
  p.nbuf = 1;
  int* blue = reinterpret_cast<int*>(base + L.blue);

  k_noalloc_tables<<<1, 256, 0, p.stream>>>(nside, lmax, p.d_cth, p.d_sth, p.d_pref,
                                            p.d_ring_i0, p.d_rfft, blue);
  FSHT_LAUNCH_CHECK();
  if ((rc = fsht_fft_tables_fill(&p, blue, f.nblue, p.stream))) return rc;
  for (int c0 = 0; c0 < nmaps; c0 += p.kchunk) {
    const int kc = nmaps - c0 < p.kchunk ? nmaps - c0 : p.kchunk;
    if ((rc = fsht_launch_ring_fft_fwd(&p, maps + (size_t)c0 * p.npix, p.npix, kc, p.d_work,
                                       p.stream)))
      return rc;
    if ((rc = fsht_launch_analysis_fp64(&p, 0, p.d_work, nullptr, alm, nullptr, nmaps, c0, kc, 0,
                                        1, p.stream)))
      return rc;
  }
  return FSHT_OK;
}
