// Plan management and the C ABI of fastsht_gb300 (include/fastsht.h).
//
// A plan replaces the reference's global Fortran module state
// (src/sht_data_module.f90, allocated by sht_data_alloc / sht_set_data,
// src/sht_data_init.f90:2-311): ring geometry, recursion seeds, ring-skip table,
// FFT tables and the phase-matrix workspace all live in one object bound to a
// CUDA stream, so independent plans can run concurrently.
#include "common.cuh"
#include "tcgen05.cuh"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

namespace {
thread_local std::string g_last_error;
// Page-locked blocks from fsht_host_alloc (start -> bytes): fsht_t2alm_host reads maps that
// lie inside one of them in place.
std::mutex g_host_mu;
std::map<const char*, size_t> g_host_blocks;
constexpr size_t kDefaultWorkspace = 16ull << 30;
constexpr size_t kDefaultWorkspaceSplit = 80ull << 30;   // 500 maps at nside 1024 in one chunk
}  // namespace

// Per-kernel event timing (enabled by fsht_profile_enable).
struct FshtProfile {
  std::vector<cudaEvent_t> pending[FSHT_KCAT_COUNT];   // begin/end pairs
  int launches[FSHT_KCAT_COUNT] = {0};
  double ms[FSHT_KCAT_COUNT] = {0.0};
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
};

namespace {
struct ProfScope {
  fsht_plan* p;
  int cat;
  cudaStream_t st;
  ProfScope(fsht_plan* pp, int c, cudaStream_t s) : p(pp), cat(c), st(s) {
    if (p->prof) {
      cudaEvent_t e = p->prof->get();
      cudaEventRecord(e, st);
      p->prof->pending[cat].push_back(e);
    }
  }
  ProfScope(fsht_plan* pp, int c) : ProfScope(pp, c, pp->stream) {}
  ~ProfScope() {
    if (p->prof) {
      cudaEvent_t e = p->prof->get();
      cudaEventRecord(e, st);
      p->prof->pending[cat].push_back(e);
    }
  }
};
}  // namespace
#define FSHT_PROF(cat) ProfScope _prof_scope_##__LINE__(p, cat)
#define FSHT_PROF_ON(cat, st) ProfScope _prof_scope_##__LINE__(p, cat, st)

int fsht_smem_limit(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> done;
  int dev = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = done[std::make_pair(dev, func)];
  if (bytes > cur) {
    FSHT_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bytes));
    cur = bytes;
  }
  return FSHT_OK;
}

void fsht_set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

namespace {

void free_plan_memory(fsht_plan* p) {
  if (!p) return;
  cudaFree(p->d_cth);
  cudaFree(p->d_sth);
  cudaFree(p->d_pref);
  cudaFree(p->d_ring_i0);
  cudaFree(p->d_rfft);
  cudaFree(p->d_chirp);
  cudaFree(p->d_rtw);
  cudaFree(p->d_bhat);
  cudaFree(p->d_tw);
  cudaFree(p->d_tw_df);
  cudaFree(p->d_chirp_df);
  cudaFree(p->d_bhat_df);
  cudaFree(p->d_rtw_df);
  cudaFree(p->d_tw16_df);
  cudaFree(p->d_work);
  cudaFree(p->d_err);
  cudaFree(p->d_ws);
  cudaFree(p->d_eb);
  cudaFree(p->d_lamtab);
  cudaFree(p->d_lam_off);
  cudaFree(p->d_lbuf);
  cudaFree(p->d_lbuf2);
  for (int i = 0; i < 6; ++i)
    if (p->ev[i]) cudaEventDestroy(p->ev[i]);
  if (p->aux) cudaStreamDestroy(p->aux);
  for (int i = 0; i < 4; ++i)
    if (p->evx[i]) cudaEventDestroy(p->evx[i]);
  if (p->xfer) cudaStreamDestroy(p->xfer);
  for (int i = 0; i < 4; ++i)
    if (p->evs[i]) cudaEventDestroy(p->evs[i]);
  if (p->aux2) cudaStreamDestroy(p->aux2);
  for (int i = 0; i < 5; ++i)
    if (p->evh[i]) cudaEventDestroy(p->evh[i]);
  if (p->hp_main) cudaStreamDestroy(p->hp_main);
  if (p->hp_aux) cudaStreamDestroy(p->hp_aux);
  if (p->hp_aux2) cudaStreamDestroy(p->hp_aux2);
  cudaFree(p->d_poltab);
  delete[] p->h_waves;
  delete[] p->h_ring_i0;
  if (p->prof) {
    for (auto& v : p->prof->pending)
      for (auto e : v) cudaEventDestroy(e);
    for (auto e : p->prof->pool) cudaEventDestroy(e);
    delete p->prof;
    p->prof = nullptr;
  }
}

// theta of the first pixel of north ring i (HEALPix pix2loc, as used through
// healpy.pix2ang at the ring start pixels, SHT.py:47-50).
double ring_theta(int ns, int i) {
  const double npix = 12.0 * ns * ns;
  const double fact2 = 4.0 / npix;
  const double fact1 = (double)(2 * ns) * fact2;
  const int ir = i + 1;
  if (ir < ns) {
    const double tmp = (double)ir * (double)ir * fact2;
    const double z = 1.0 - tmp;
    if (z > 0.99) return std::atan2(std::sqrt(tmp * (2.0 - tmp)), z);
    return std::acos(z);
  }
  const double z = (double)(2 * ns - ir) * fact1;
  return std::acos(z);
}

int check_plan(const fsht_plan* p) {
  if (!p) {
    fsht_set_error("null plan");
    return FSHT_EINVAL;
  }
  return FSHT_OK;
}

size_t per_map_buffer_bytes(const fsht_plan* p) {
  return (size_t)(p->lmax + 1) * p->nnorth * 2 * sizeof(double2);
}

double2* work_buf(fsht_plan* p, int b, int kc) {
  return p->d_work + (size_t)b * kc * (size_t)(p->lmax + 1) * p->nnorth * 2;
}

int check_call(fsht_plan* p, int nmaps, const void* a, const void* b) {
  int rc = check_plan(p);
  if (rc) return rc;
  if (p->kchunk < 1 || !p->d_work) {
    fsht_set_error("this plan holds no workspace (created with FSHT_FLAG_TABLES_ONLY)");
    return FSHT_EINVAL;
  }
  if (nmaps < 1 || nmaps > p->nmaps_max) {
    fsht_set_error("nmaps = %d outside [1, %d] of this plan", nmaps, p->nmaps_max);
    return FSHT_EINVAL;
  }
  if (!a || !b) {
    fsht_set_error("null array pointer");
    return FSHT_EINVAL;
  }
  return FSHT_OK;
}

int need_bufs(fsht_plan* p, int nb) {
  if (nb > p->nbuf) {
    fsht_set_error("this call needs %d workspace buffers but the plan holds %d "
                   "(create it with FSHT_FLAG_POL / FSHT_FLAG_ITER)", nb, p->nbuf);
    return FSHT_EINVAL;
  }
  return FSHT_OK;
}

}  // namespace

extern "C" {

int fsht_last_error(char* buf, size_t len) {
  if (buf && len) {
    size_t n = g_last_error.size() < len - 1 ? g_last_error.size() : len - 1;
    memcpy(buf, g_last_error.data(), n);
    buf[n] = 0;
  }
  return (int)g_last_error.size();
}

int fsht_plan_create(int nside, int lmax, int nmaps_max, int flags, int precision,
                     size_t workspace_limit_bytes, void* stream, fsht_plan** out) {
  if (!out) {
    fsht_set_error("null output pointer");
    return FSHT_EINVAL;
  }
  *out = nullptr;
  if (nside < 1 || nside > 2048 || (nside & (nside - 1))) {
    fsht_set_error("nside = %d: must be a power of two in [1, 2048]", nside);
    return nside > 2048 && !(nside & (nside - 1)) ? FSHT_EUNSUPPORTED : FSHT_EINVAL;
  }
  if (lmax < 0 || lmax > 4 * nside) {
    fsht_set_error("lmax = %d outside [0, 4*nside = %d]", lmax, 4 * nside);
    return FSHT_EINVAL;
  }
  if (nmaps_max < 1) {
    fsht_set_error("nmaps_max = %d must be >= 1", nmaps_max);
    return FSHT_EINVAL;
  }
  if (precision != FSHT_PREC_FP64 && precision != FSHT_PREC_SPLIT) {
    fsht_set_error("precision %d: use FSHT_PREC_FP64 or FSHT_PREC_SPLIT", precision);
    return FSHT_EUNSUPPORTED;
  }
  fsht_plan* p = new (std::nothrow) fsht_plan();
  if (!p) {
    fsht_set_error("host allocation failed");
    return FSHT_ENOMEM;
  }
  memset(p, 0, sizeof(*p));
  p->nside = nside;
  p->lmax = lmax;
  p->nring = 4 * nside - 1;
  p->nnorth = 2 * nside;
  p->npix = 12LL * nside * nside;
  p->nmaps_max = nmaps_max;
  p->pol = (flags & FSHT_FLAG_POL) ? 1 : 0;
  p->precision = precision;
  p->stream = (cudaStream_t)stream;
  p->pa = 4.0 * M_PI / (double)p->npix;
  p->nbuf = ((flags & FSHT_FLAG_POL) ? 2 : 1) * ((flags & FSHT_FLAG_ITER) ? 2 : 1);
  p->h_ring_i0 = new (std::nothrow) int[lmax + 1];
  int rc = FSHT_OK;
  auto fail = [&](int code) {
    free_plan_memory(p);
    delete p;
    return code;
  };
  if (!p->h_ring_i0) {
    fsht_set_error("host allocation failed");
    return fail(FSHT_ENOMEM);
  }
  // ---- ring tables
  const int nn = p->nnorth;
  std::vector<double> cth(nn), sth(nn), pref(lmax + 1);
  for (int i = 0; i < nn; ++i) {
    const double th = ring_theta(nside, i);
    cth[i] = std::cos(th);
    sth[i] = std::sin(th);
  }
  // diag_fac(m) = prod_{k<=m} (2k+1)/(2k)  (set_out_of_loop_constants,
  // src/sht_data_init.f90:414-418); seed prefactor sqrt(diag_fac/4/pi)
  // (get_plm_recursive.f90:46)
  double df = 1.0;
  for (int m = 0; m <= lmax; ++m) {
    if (m > 0) df = df * (2 * m + 1) / 2 / m;
    pref[m] = std::sqrt(df / 4 / M_PI);
  }
  auto dalloc = [&](void** ptr, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
      fsht_set_error("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? FSHT_ENOMEM : FSHT_ECUDA;
    }
    return FSHT_OK;
  };
  if ((rc = dalloc((void**)&p->d_cth, sizeof(double) * nn))) return fail(rc);
  if ((rc = dalloc((void**)&p->d_sth, sizeof(double) * nn))) return fail(rc);
  if ((rc = dalloc((void**)&p->d_pref, sizeof(double) * (lmax + 1)))) return fail(rc);
  if ((rc = dalloc((void**)&p->d_ring_i0, sizeof(int) * (lmax + 1)))) return fail(rc);
  cudaError_t ce;
  if ((ce = cudaMemcpyAsync(p->d_cth, cth.data(), sizeof(double) * nn, cudaMemcpyHostToDevice,
                            p->stream)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(p->d_sth, sth.data(), sizeof(double) * nn, cudaMemcpyHostToDevice,
                            p->stream)) != cudaSuccess ||
      (ce = cudaMemcpyAsync(p->d_pref, pref.data(), sizeof(double) * (lmax + 1),
                            cudaMemcpyHostToDevice, p->stream)) != cudaSuccess) {
    fsht_set_error("table upload: %s", cudaGetErrorString(ce));
    return fail(FSHT_ECUDA);
  }
  if ((rc = fsht_launch_ring_skip(p, p->stream))) return fail(rc);
  if ((rc = fsht_fft_tables_init(p))) return fail(rc);
  if (precision == FSHT_PREC_SPLIT && (rc = fsht_fft_df_tables_init(p))) return fail(rc);
  if (precision == FSHT_PREC_SPLIT && (rc = fsht_split_tables_init(p))) return fail(rc);
  if (precision == FSHT_PREC_SPLIT && p->pol && (rc = fsht_split_pol_tables_init(p)))
    return fail(rc);
  // ---- workspace: nbuf phase matrices of kchunk maps (+ the sliced copy for the
  // split form, sized in groups of 128 maps)
  const size_t limit = workspace_limit_bytes
                           ? workspace_limit_bytes
                           : (precision == FSHT_PREC_SPLIT ? kDefaultWorkspaceSplit : kDefaultWorkspace);
  const size_t per_map = per_map_buffer_bytes(p) * p->nbuf;
  // digit-tile buffers of the split form: two waves in flight of T, or of Q and U (four)
  const size_t f_ws = p->pol ? 4 : 2;
  auto need = [&](size_t k) -> size_t {
    size_t b = per_map * k;
    if (precision == FSHT_PREC_SPLIT)   // digit tiles and their exponents, two lambda buffers
      b += f_ws * (fsht_split_ws_bytes(p, (int)k) + fsht_split_eb_bytes(p, (int)k)) +
           2 * p->lbuf_bytes;
    return b;
  };
  const bool tables_only = (flags & FSHT_FLAG_TABLES_ONLY) != 0;
  size_t kc = (size_t)nmaps_max;
  while (kc > 1 && need(kc) > limit) kc = (kc > 128 && kc % 128) ? kc - kc % 128 : kc - (kc > 128 ? 128 : 1);
  if (!tables_only && need(kc) > limit) {
    fsht_set_error("workspace limit %zu bytes is below one map's %zu bytes", limit, need(1));
    return fail(FSHT_EINVAL);
  }
  p->kchunk = tables_only ? 0 : (int)kc;
  p->work_bytes = tables_only ? 0 : per_map * kc;
  if (!tables_only && (rc = dalloc((void**)&p->d_work, p->work_bytes))) return fail(rc);
  if ((rc = dalloc((void**)&p->d_err, sizeof(int)))) return fail(rc);
  if ((ce = cudaMemsetAsync(p->d_err, 0, sizeof(int), p->stream)) != cudaSuccess) {
    fsht_set_error("memset: %s", cudaGetErrorString(ce));
    return fail(FSHT_ECUDA);
  }
  if (precision == FSHT_PREC_SPLIT && !tables_only) {
    const size_t f = f_ws;
    p->ws_bytes = f * fsht_split_ws_bytes(p, p->kchunk);
    if ((rc = dalloc((void**)&p->d_ws, p->ws_bytes))) return fail(rc);
    if ((rc = dalloc((void**)&p->d_eb, f * fsht_split_eb_bytes(p, p->kchunk)))) return fail(rc);
    if ((rc = dalloc((void**)&p->d_lbuf, p->lbuf_bytes))) return fail(rc);
    if ((rc = dalloc((void**)&p->d_lbuf2, p->lbuf_bytes))) return fail(rc);
    if ((ce = cudaStreamCreateWithFlags(&p->aux, cudaStreamNonBlocking)) != cudaSuccess) {
      fsht_set_error("auxiliary stream: %s", cudaGetErrorString(ce));
      return fail(FSHT_ECUDA);
    }
    for (int i = 0; i < 6; ++i) {
      if ((ce = cudaEventCreateWithFlags(&p->ev[i], cudaEventDisableTiming)) != cudaSuccess) {
        fsht_set_error("event: %s", cudaGetErrorString(ce));
        return fail(FSHT_ECUDA);
      }
    }
    if ((ce = cudaStreamCreateWithFlags(&p->aux2, cudaStreamNonBlocking)) != cudaSuccess) {
      fsht_set_error("auxiliary stream: %s", cudaGetErrorString(ce));
      return fail(FSHT_ECUDA);
    }
    for (int i = 0; i < 4; ++i) {
      if ((ce = cudaEventCreateWithFlags(&p->evs[i], cudaEventDisableTiming)) != cudaSuccess) {
        fsht_set_error("event: %s", cudaGetErrorString(ce));
        return fail(FSHT_ECUDA);
      }
    }
    int least = 0, greatest = 0;
    if ((ce = cudaDeviceGetStreamPriorityRange(&least, &greatest)) != cudaSuccess ||
        (ce = cudaStreamCreateWithPriority(&p->hp_main, cudaStreamNonBlocking, greatest)) !=
            cudaSuccess ||
        (ce = cudaStreamCreateWithPriority(&p->hp_aux, cudaStreamNonBlocking, greatest)) !=
            cudaSuccess ||
        (ce = cudaStreamCreateWithPriority(&p->hp_aux2, cudaStreamNonBlocking, greatest)) !=
            cudaSuccess) {
      fsht_set_error("high-priority stream: %s", cudaGetErrorString(ce));
      return fail(FSHT_ECUDA);
    }
    for (int i = 0; i < 5; ++i) {
      if ((ce = cudaEventCreateWithFlags(&p->evh[i], cudaEventDisableTiming)) != cudaSuccess) {
        fsht_set_error("event: %s", cudaGetErrorString(ce));
        return fail(FSHT_ECUDA);
      }
    }
  }
  if (!tables_only) {
    if ((ce = cudaStreamCreateWithFlags(&p->xfer, cudaStreamNonBlocking)) != cudaSuccess) {
      fsht_set_error("copy stream: %s", cudaGetErrorString(ce));
      return fail(FSHT_ECUDA);
    }
    for (int i = 0; i < 4; ++i) {
      if ((ce = cudaEventCreateWithFlags(&p->evx[i], cudaEventDisableTiming)) != cudaSuccess) {
        fsht_set_error("event: %s", cudaGetErrorString(ce));
        return fail(FSHT_ECUDA);
      }
    }
  }
  if ((ce = cudaStreamSynchronize(p->stream)) != cudaSuccess) {
    fsht_set_error("plan setup: %s", cudaGetErrorString(ce));
    return fail(FSHT_ECUDA);
  }
  *out = p;
  return FSHT_OK;
}

int fsht_plan_destroy(fsht_plan* p) {
  if (!p) return FSHT_OK;
  cudaStreamSynchronize(p->stream);
  free_plan_memory(p);
  delete p;
  return FSHT_OK;
}

int fsht_plan_set_stream(fsht_plan* p, void* stream) {
  FSHT_TRY(check_plan(p));
  p->stream = (cudaStream_t)stream;
  return FSHT_OK;
}

int fsht_plan_info(const fsht_plan* p, size_t* device_bytes, int* maps_per_chunk) {
  FSHT_TRY(check_plan(p));
  if (device_bytes) {
    size_t b = p->work_bytes + p->ws_bytes + p->lbuf_bytes * (p->aux ? 2 : 1);
    b += sizeof(double) * (2 * p->nnorth + p->lmax + 1) + sizeof(int) * (p->lmax + 1);
    *device_bytes = b;
  }
  if (maps_per_chunk) *maps_per_chunk = p->kchunk;
  return FSHT_OK;
}

int fsht_plan_ring_skip(const fsht_plan* p, int* out) {
  FSHT_TRY(check_plan(p));
  if (!out) {
    fsht_set_error("null output");
    return FSHT_EINVAL;
  }
  memcpy(out, p->h_ring_i0, sizeof(int) * (p->lmax + 1));
  return FSHT_OK;
}

int fsht_profile_enable(fsht_plan* p, int on) {
  FSHT_TRY(check_plan(p));
  if (on && !p->prof) p->prof = new (std::nothrow) FshtProfile();
  if (on && !p->prof) {
    fsht_set_error("host allocation failed");
    return FSHT_ENOMEM;
  }
  if (!on && p->prof) {
    cudaStreamSynchronize(p->stream);
    for (auto& v : p->prof->pending)
      for (auto e : v) cudaEventDestroy(e);
    for (auto e : p->prof->pool) cudaEventDestroy(e);
    delete p->prof;
    p->prof = nullptr;
  }
  return FSHT_OK;
}

int fsht_profile_read(fsht_plan* p, int ncat, int* launches, double* total_ms) {
  FSHT_TRY(check_plan(p));
  if (!p->prof) {
    fsht_set_error("profiling is not enabled on this plan");
    return FSHT_EINVAL;
  }
  FSHT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  FshtProfile& pr = *p->prof;
  for (int c = 0; c < FSHT_KCAT_COUNT; ++c) {
    auto& v = pr.pending[c];
    for (size_t j = 0; j + 1 < v.size(); j += 2) {
      float ms = 0.f;
      FSHT_CUDA_TRY(cudaEventElapsedTime(&ms, v[j], v[j + 1]));
      pr.ms[c] += ms;
      pr.launches[c] += 1;
    }
    for (auto e : v) pr.pool.push_back(e);
    v.clear();
    if (c < ncat) {
      if (launches) launches[c] = pr.launches[c];
      if (total_ms) total_ms[c] = pr.ms[c];
    }
    pr.launches[c] = 0;
    pr.ms[c] = 0.0;
  }
  return FSHT_OK;
}

int fsht_plan_sync(fsht_plan* p) {
  FSHT_TRY(check_plan(p));
  FSHT_CUDA_TRY(cudaStreamSynchronize(p->stream));
  return fsht_plan_check(p);
}

int fsht_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) {
    fsht_set_error("host_alloc: null output pointer");
    return FSHT_EINVAL;
  }
  *ptr = nullptr;
  const size_t n = bytes > 0 ? bytes : 1;
  cudaError_t e = cudaHostAlloc(ptr, n, cudaHostAllocPortable | cudaHostAllocMapped);
  if (e != cudaSuccess) {
    fsht_set_error("cudaHostAlloc(%zu): %s", bytes, cudaGetErrorString(e));
    *ptr = nullptr;
    return e == cudaErrorMemoryAllocation ? FSHT_ENOMEM : FSHT_ECUDA;
  }
  std::lock_guard<std::mutex> lk(g_host_mu);
  g_host_blocks[static_cast<const char*>(*ptr)] = n;
  return FSHT_OK;
}

int fsht_host_free(void* ptr) {
  if (!ptr) return FSHT_OK;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    g_host_blocks.erase(static_cast<const char*>(ptr));
  }
  FSHT_CUDA_TRY(cudaFreeHost(ptr));
  return FSHT_OK;
}

namespace {
// The device address of host bytes [ptr, ptr + bytes) when they lie inside one
// fsht_host_alloc block (mapped into the device's address space), else null.
const double* host_direct(const void* ptr, size_t bytes) {
  const char* c = static_cast<const char*>(ptr);
  const char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = g_host_blocks.upper_bound(c);
    if (it == g_host_blocks.begin()) return nullptr;
    --it;
    const size_t off = (size_t)(c - it->first);
    if (off >= it->second || bytes > it->second - off) return nullptr;
    base = it->first;
  }
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, const_cast<char*>(base), 0) != cudaSuccess || !d) {
    cudaGetLastError();   // not mapped for this device: the caller stages the maps
    return nullptr;
  }
  return reinterpret_cast<const double*>(static_cast<const char*>(d) + (c - base));
}
}  // namespace

int fsht_host_mapped(const void* ptr, size_t bytes, int* mapped) {
  if (!mapped) {
    fsht_set_error("host_mapped: null output pointer");
    return FSHT_EINVAL;
  }
  *mapped = (ptr && host_direct(ptr, bytes)) ? 1 : 0;
  return FSHT_OK;
}

int fsht_plan_set_host_read(fsht_plan* p, int direct) {
  FSHT_TRY(check_plan(p));
  if (direct < 0 || direct > 2) {
    fsht_set_error("host read mode %d: 0 (staged), 1 (in place) or 2 (in place, in chunks)",
                   direct);
    return FSHT_EINVAL;
  }
  p->host_staged = direct ? 0 : 1;
  p->host_chunked = direct == 2 ? 1 : 0;
  return FSHT_OK;
}

int fsht_plan_check(fsht_plan* p) {
  FSHT_TRY(check_plan(p));
  int err = 0;
  FSHT_CUDA_TRY(cudaMemcpy(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (err) {
    FSHT_CUDA_TRY(cudaMemset(p->d_err, 0, sizeof(int)));
    if (err & tc::kErrTimeout) {
      fsht_set_error("a bounded device-side wait expired (error word %d); results are invalid",
                     err);
      return FSHT_ETIMEOUT;
    }
    fsht_set_error("a value fell outside its digit scale in the split form (error word %d: "
                   "non-finite input?); results are invalid", err);
    return FSHT_ERANGE;
  }
  return FSHT_OK;
}

// ----------------------------------------------------------------- split form
// Wave pipeline of the lambda-digit tiles.  The tiles depend on the plan only, so a plan
// that owns its workspace computes them on its auxiliary stream two waves ahead of the
// contraction, alternating between two staging buffers: the recursion (FP64 pipe) overlaps
// the ring FFT (FP32 pipe; wave 0 and 1 start before it) and the slicing / tensor-core
// contraction of earlier waves.  Events order each contraction after its tiles and each
// refill after the contraction that read the buffer.  Job views of table-only plans (the
// batched and serving forms, which already run several jobs concurrently) have no
// auxiliary stream and run the kernels in turn on one stream.
typedef int (*LamLaunch)(fsht_plan*, int, unsigned char*, cudaStream_t);
enum { kEvFork = 0, kEvJoin = 1, kEvTiles = 2, kEvDone = 4 };

static unsigned char* lam_buf(fsht_plan* p, int w) {
  return (p->aux && (w & 1)) ? p->d_lbuf2 : p->d_lbuf;
}

static int lam_ahead(fsht_plan* p, LamLaunch f, int w) {
  if (w >= 2) FSHT_CUDA_TRY(cudaStreamWaitEvent(p->aux, p->ev[kEvDone + (w & 1)], 0));
  {
    FSHT_PROF_ON(FSHT_KCAT_LAMBDA, p->aux);
    FSHT_TRY(f(p, w, lam_buf(p, w), p->aux));
  }
  FSHT_CUDA_TRY(cudaEventRecord(p->ev[kEvTiles + (w & 1)], p->aux));
  return FSHT_OK;
}

// Forks the auxiliary stream off the plan's stream and starts waves 0 and 1.
static int lam_start(fsht_plan* p, LamLaunch f) {
  if (!p->aux) return FSHT_OK;
  FSHT_CUDA_TRY(cudaEventRecord(p->ev[kEvFork], p->stream));
  FSHT_CUDA_TRY(cudaStreamWaitEvent(p->aux, p->ev[kEvFork], 0));
  FSHT_TRY(lam_ahead(p, f, 0));
  if (p->nwaves > 1) FSHT_TRY(lam_ahead(p, f, 1));
  return FSHT_OK;
}

// Before wave w's contraction: its tiles, in the returned buffer, are ready for the plan's
// stream (computed there now when the plan has no auxiliary stream).
static int lam_ready(fsht_plan* p, LamLaunch f, int w, unsigned char** buf) {
  if (!p->aux) {
    FSHT_PROF(FSHT_KCAT_LAMBDA);
    FSHT_TRY(f(p, w, p->d_lbuf, p->stream));
    *buf = p->d_lbuf;
    return FSHT_OK;
  }
  FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->ev[kEvTiles + (w & 1)], 0));
  *buf = lam_buf(p, w);
  return FSHT_OK;
}

// After wave w's contraction: its buffer may be refilled with wave w + 2.
static int lam_done(fsht_plan* p, LamLaunch f, int w) {
  if (!p->aux) return FSHT_OK;
  FSHT_CUDA_TRY(cudaEventRecord(p->ev[kEvDone + (w & 1)], p->stream));
  if (w + 2 < p->nwaves) FSHT_TRY(lam_ahead(p, f, w + 2));
  return FSHT_OK;
}

// Joins the auxiliary stream back into the plan's stream.
static int lam_finish(fsht_plan* p) {
  if (!p->aux) return FSHT_OK;
  FSHT_CUDA_TRY(cudaEventRecord(p->ev[kEvJoin], p->aux));
  FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->ev[kEvJoin], 0));
  return FSHT_OK;
}

// Host-buffer transfers of fsht_t2alm_host on the plan's copy stream: the maps land in
// sub-batches, each forward-transformed as soon as it is on the device, and alm columns go
// back as soon as every order they hold is final (after each wave of the split form when
// niter = 0, else at the end of the chunk).  Column c holds Re a_lm of m = c and Im a_lm of
// m = lmax + 1 - c, so it is final once both orders are.
struct HostXfer {
  const double* hmaps;
  const double* direct;   // device address of hmaps when the FFT reads them in place, or null
  double* halm;
  std::vector<char> mdone, cdone;
};

static int xfer_wait_main(fsht_plan* p, int ev) {
  FSHT_CUDA_TRY(cudaEventRecord(p->evx[ev], p->stream));
  FSHT_CUDA_TRY(cudaStreamWaitEvent(p->xfer, p->evx[ev], 0));
  return FSHT_OK;
}

static int xfer_join(fsht_plan* p) {
  FSHT_CUDA_TRY(cudaEventRecord(p->evx[3], p->xfer));
  FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->evx[3], 0));
  return FSHT_OK;
}

// Orders of pair-order range [q0, q1) are final in the device alm of maps [c0, c0 + kc):
// copy the columns that became complete (runs of adjacent columns as 2D copies).
static int xfer_orders_done(fsht_plan* p, HostXfer& x, const double* dalm, int nmaps, int q0,
                            int q1, int c0, int kc) {
  const int lmax = p->lmax;
  for (int q = q0; q < q1; ++q) x.mdone[(q & 1) ? lmax - (q >> 1) : (q >> 1)] = 1;
  FSHT_TRY(xfer_wait_main(p, 2));
  const size_t L1 = (size_t)lmax + 1, pitch = sizeof(double) * nmaps;
  int c = 0;
  while (c <= lmax) {
    auto ready = [&](int cc) {
      return !x.cdone[cc] && x.mdone[cc] && (cc == 0 || x.mdone[lmax + 1 - cc]);
    };
    if (!ready(c)) {
      ++c;
      continue;
    }
    int e = c;
    while (e <= lmax && ready(e)) x.cdone[e++] = 1;
    const size_t off = (size_t)c * L1 * nmaps + c0;
    FSHT_CUDA_TRY(cudaMemcpy2DAsync(x.halm + off, pitch, dalm + off, pitch,
                                    sizeof(double) * kc, (size_t)(e - c) * L1,
                                    cudaMemcpyDeviceToHost, p->xfer));
    c = e;
  }
  return FSHT_OK;
}

// One chunk's split-precision analysis of the {S, D} matrix W into alm (added when
// accumulate), and synthesis of alm into W = {G_N, G_S}.  started: lam_start already ran
// (before the FFT).  hx: copy each wave's finished alm columns to the host.
static int split_analysis(fsht_plan* p, const double2* W, double* alm, int nmaps, int c0, int kc,
                          int accumulate, bool started = false, HostXfer* hx = nullptr) {
  // every alm element of the chunk is written by exactly one unit of the contraction (its
  // first ring part stores, later parts add), so alm needs no clearing
  if (!started) FSHT_TRY(lam_start(p, fsht_launch_split_lambda));
  // Slicing runs one wave ahead on the second auxiliary stream, alternating between the two
  // halves of d_ws / d_eb: the HBM-bound slicing of wave w + 1 shares the SMs with the
  // tensor-core contraction of wave w.  The slice of wave w + 1 waits for the contraction of
  // wave w - 1 (the "contraction done" events of the lambda pipeline), the contraction of
  // wave w for its slice.
  const bool ahead = p->aux2 != nullptr && p->aux != nullptr;
  const size_t ws1 = fsht_split_ws_bytes(p, kc);
  const size_t eb1 = fsht_split_eb_bytes(p, kc) / sizeof(int);
  auto ws_of = [&](int w) { return p->d_ws + (ahead ? (size_t)(w & 1) * ws1 : 0); };
  auto eb_of = [&](int w) { return p->d_eb + (ahead ? (size_t)(w & 1) * eb1 : 0); };
  auto slice_on = [&](int w, cudaStream_t st) -> int {
    FSHT_PROF_ON(FSHT_KCAT_SLICE, st);
    return fsht_launch_split_slice(p, w, W, ws_of(w), eb_of(w), kc, st);
  };
  if (ahead) {
    FSHT_CUDA_TRY(cudaEventRecord(p->evs[0], p->stream));
    FSHT_CUDA_TRY(cudaStreamWaitEvent(p->aux2, p->evs[0], 0));
    FSHT_TRY(slice_on(0, p->aux2));
    FSHT_CUDA_TRY(cudaEventRecord(p->evs[2], p->aux2));
  }
  for (int w = 0; w < p->nwaves; ++w) {
    if (!ahead) {
      FSHT_TRY(slice_on(w, p->stream));
    } else {
      if (w + 1 < p->nwaves) {
        if (w >= 1)
          FSHT_CUDA_TRY(cudaStreamWaitEvent(p->aux2, p->ev[kEvDone + ((w + 1) & 1)], 0));
        FSHT_TRY(slice_on(w + 1, p->aux2));
        FSHT_CUDA_TRY(cudaEventRecord(p->evs[2 + ((w + 1) & 1)], p->aux2));
      }
      FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->evs[2 + (w & 1)], 0));
    }
    unsigned char* lb = nullptr;
    FSHT_TRY(lam_ready(p, fsht_launch_split_lambda, w, &lb));
    {
      FSHT_PROF(FSHT_KCAT_ANALYSIS);
      FSHT_TRY(fsht_launch_split_gemm(p, w, ws_of(w), eb_of(w), lb, alm, nmaps, c0, kc,
                                      accumulate, p->stream));
    }
    FSHT_TRY(lam_done(p, fsht_launch_split_lambda, w));
    if (hx) {
      int q0, q1;
      fsht_split_wave_range(p, w, &q0, &q1);
      FSHT_TRY(xfer_orders_done(p, *hx, alm, nmaps, q0, q1, c0, kc));
    }
  }
  if (ahead) {
    FSHT_CUDA_TRY(cudaEventRecord(p->evs[1], p->aux2));
    FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->evs[1], 0));
  }
  return lam_finish(p);
}

static int split_synthesis(fsht_plan* p, const double* alm, double2* W, int nmaps, int c0,
                           int kc) {
  // the first even-l pass of every unit stores G_N and G_S, later passes add: no clearing
  FSHT_TRY(lam_start(p, fsht_launch_split_lambdaT));
  for (int w = 0; w < p->nwaves; ++w) {
    {
      FSHT_PROF(FSHT_KCAT_SLICE);
      FSHT_TRY(fsht_launch_split_slice_alm(p, w, alm, p->d_ws, p->d_eb, nmaps, c0, kc,
                                           p->stream));
    }
    unsigned char* lb = nullptr;
    FSHT_TRY(lam_ready(p, fsht_launch_split_lambdaT, w, &lb));
    {
      FSHT_PROF(FSHT_KCAT_SYNTHESIS);
      FSHT_TRY(fsht_launch_split_synth(p, w, p->d_ws, p->d_eb, lb, W, kc, p->stream));
    }
    FSHT_TRY(lam_done(p, fsht_launch_split_lambdaT, w));
  }
  return lam_finish(p);
}

int fsht_run_stage(fsht_plan* p, int stage, const void* in, void* out, int nmaps) {
  FSHT_TRY(check_call(p, nmaps, in, out));
  if (nmaps > p->kchunk) {
    fsht_set_error("run_stage: nmaps %d above maps_per_chunk %d", nmaps, p->kchunk);
    return FSHT_EINVAL;
  }
  switch (stage) {
    case FSHT_STAGE_FFT_FWD:
      return fsht_launch_ring_fft_fwd(p, (const double*)in, p->npix, nmaps, (double2*)out,
                                      p->stream);
    case FSHT_STAGE_ANALYSIS:
      if (p->precision == FSHT_PREC_SPLIT)
        return split_analysis(p, (const double2*)in, (double*)out, nmaps, 0, nmaps, 0);
      return fsht_launch_analysis_fp64(p, 0, (const double2*)in, nullptr, (double*)out, nullptr,
                                       nmaps, 0, nmaps, 0, 1, p->stream);
    case FSHT_STAGE_SYNTHESIS:
      if (p->precision == FSHT_PREC_SPLIT)
        return split_synthesis(p, (const double*)in, (double2*)out, nmaps, 0, nmaps);
      return fsht_launch_synthesis_fp64(p, 0, (const double*)in, nullptr, (double2*)out, nullptr,
                                        nmaps, 0, nmaps, p->stream);
    case FSHT_STAGE_FFT_INV:
      return fsht_launch_ring_fft_inv(p, (const double2*)in, (double*)out, p->npix, nmaps,
                                      p->stream);
    default:
      fsht_set_error("unknown stage %d", stage);
      return FSHT_EINVAL;
  }
}

// ----------------------------------------------------------------- temperature
// SMs the persistent GEMM leaves to the next chunk's forward FFT in the chunked host route:
// reading maps in place is bound by the host link, which about two dozen SMs keep busy.
constexpr int kFftSms = 24;

// Maps per chunk of the chunked host route (a multiple of the 64-map tile), or 0 when the
// route does not apply: the split form without iterations, maps read in place, at least two
// chunks' phase matrices in the workspace.
static int host_chunk_maps(const fsht_plan* p, int nmaps, int niter, const HostXfer* hx) {
  if (!hx || !hx->direct || !p->host_chunked || niter != 0 ||
      p->precision != FSHT_PREC_SPLIT || !p->hp_main || nmaps < 128)
    return 0;
  const int nch = nmaps >= 256 ? 4 : 2;
  int kc = (nmaps + nch - 1) / nch;
  kc = (kc + 63) / 64 * 64;
  return 2 * kc <= p->kchunk ? kc : 0;
}

static void swap_hp(fsht_plan* p) {
  std::swap(p->stream, p->hp_main);
  std::swap(p->aux, p->hp_aux);
  std::swap(p->aux2, p->hp_aux2);
}

// fsht_t2alm_host, split form, maps read in place: chunks of kc maps whose forward FFT reads
// the host link on the plan's stream while the previous chunk's contraction (recursion, slicing,
// tensor-core GEMM, alm copies back) runs on high-priority copies of the plan's streams, two
// phase-matrix buffers alternating.  The link-bound FFT needs few SMs: the GEMM's persistent
// grid leaves it kFftSms while a later chunk is pending, and the contraction's kernels, at the
// higher priority, take the others as the FFT's thread blocks retire.  The recursion runs once
// per chunk (its digit tiles are not kept between chunks).
static int t2alm_host_chunked(fsht_plan* p, double* alm, int nmaps, int kc, HostXfer* hx) {
  const int nch = (nmaps + kc - 1) / kc;
  const size_t per_map = per_map_buffer_bytes(p) / sizeof(double2);
  double2* Wb[2] = {p->d_work, p->d_work + per_map * kc};
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  FSHT_CUDA_TRY(cudaEventRecord(p->evh[0], p->stream));
  FSHT_CUDA_TRY(cudaStreamWaitEvent(p->hp_main, p->evh[0], 0));
  for (int c = 0; c < nch; ++c) {
    const int c0 = c * kc, n = nmaps - c0 < kc ? nmaps - c0 : kc, b = c & 1;
    // buffer b is free once the contraction of chunk c - 2 has read it
    if (c >= 2) FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->evh[3 + b], 0));
    {
      FSHT_PROF(FSHT_KCAT_FFT_FWD);
      FSHT_TRY(fsht_launch_ring_fft_fwd(p, hx->direct + (size_t)c0 * p->npix, p->npix, n, Wb[b],
                                        p->stream));
    }
    FSHT_CUDA_TRY(cudaEventRecord(p->evh[1 + b], p->stream));
    swap_hp(p);
    p->gemm_ctas = (c + 1 < nch && nsm > 2 * kFftSms) ? nsm - kFftSms : 0;
    hx->mdone.assign(p->lmax + 1, 0);
    hx->cdone.assign(p->lmax + 1, 0);
    int rc = cudaStreamWaitEvent(p->stream, p->evh[1 + b], 0) == cudaSuccess ? FSHT_OK
                                                                               : FSHT_ECUDA;
    if (!rc) rc = split_analysis(p, Wb[b], alm, nmaps, c0, n, 0, false, hx);
    if (!rc) rc = xfer_orders_done(p, *hx, alm, nmaps, 0, p->lmax + 1, c0, n);
    if (!rc && cudaEventRecord(p->evh[3 + b], p->stream) != cudaSuccess) rc = FSHT_ECUDA;
    p->gemm_ctas = 0;
    swap_hp(p);
    if (rc) {
      if (rc == FSHT_ECUDA) fsht_set_error("chunked host route: CUDA error");
      return rc;
    }
  }
  // the plan's stream resumes after the last contraction
  FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->evh[3 + ((nch - 1) & 1)], 0));
  return FSHT_OK;
}

// hx: the maps come from host memory (copied in sub-batches that the FFT consumes as they
// land) and the alm go back to it; null: device buffers only.
static int t2alm_impl(fsht_plan* p, const double* maps, double* alm, int nmaps, int niter,
                      int method, HostXfer* hx) {
  FSHT_TRY(need_bufs(p, niter > 0 ? 2 : 1));
  const bool split = p->precision == FSHT_PREC_SPLIT;
  if (hx) FSHT_TRY(xfer_wait_main(p, 0));   // the device buffers' earlier users are done
  if (const int kc = host_chunk_maps(p, nmaps, niter, hx)) {
    FSHT_TRY(t2alm_host_chunked(p, alm, nmaps, kc, hx));
    return xfer_join(p);
  }
  for (int c0 = 0; c0 < nmaps; c0 += p->kchunk) {
    const int kc = nmaps - c0 < p->kchunk ? nmaps - c0 : p->kchunk;
    double2* W0 = work_buf(p, 0, kc);
    if (hx) {
      hx->mdone.assign(p->lmax + 1, 0);
      hx->cdone.assign(p->lmax + 1, 0);
    }
    // the first lambda tiles are computed on the auxiliary stream during the FFT
    if (split) FSHT_TRY(lam_start(p, fsht_launch_split_lambda));
    // the chunk's maps as the FFT reads them: device buffer, or host memory read in place
    const double* cmaps = (hx && hx->direct ? hx->direct : maps) + (size_t)c0 * p->npix;
    if (!hx || hx->direct) {
      FSHT_PROF(FSHT_KCAT_FFT_FWD);
      // (page-locked maps mapped into the device's address space are read over the host link
      // as the transform goes, every value once, with no staging copy)
      FSHT_TRY(fsht_launch_ring_fft_fwd(p, cmaps, p->npix, kc, W0, p->stream));
    } else {
      // sub-batches of a multiple of 16 maps, at most 8
      int kb = (kc + 7) / 8;
      kb = (kb + 15) / 16 * 16;
      for (int k0 = 0; k0 < kc; k0 += kb) {
        const int cnt = kc - k0 < kb ? kc - k0 : kb;
        const size_t off = (size_t)(c0 + k0) * p->npix;
        FSHT_CUDA_TRY(cudaMemcpyAsync(const_cast<double*>(maps) + off, hx->hmaps + off,
                                      sizeof(double) * p->npix * cnt, cudaMemcpyHostToDevice,
                                      p->xfer));
        FSHT_CUDA_TRY(cudaEventRecord(p->evx[1], p->xfer));
        FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->evx[1], 0));
        FSHT_PROF(FSHT_KCAT_FFT_FWD);
        FSHT_TRY(fsht_launch_ring_fft_fwd_part(p, cmaps, p->npix, kc, k0, cnt, W0, p->stream));
      }
    }
    if (split) {
      FSHT_TRY(split_analysis(p, W0, alm, nmaps, c0, kc, 0, true, niter == 0 ? hx : nullptr));
      // Jacobi refinement: FP64 Fourier-space residual of a split synthesis, analysed
      // in split precision and added
      for (int it = 0; it < niter; ++it) {
        double2* W1 = work_buf(p, 1, kc);
        FSHT_TRY(split_synthesis(p, alm, W1, nmaps, c0, kc));
        {
          FSHT_PROF(FSHT_KCAT_RESIDUAL);
          FSHT_TRY(fsht_launch_fourier_residual(p, W0, W1, kc, method, p->stream));
        }
        FSHT_TRY(split_analysis(p, W1, alm, nmaps, c0, kc, 1));
      }
    } else {
      double2* W1 = work_buf(p, 1, kc);
      {
        FSHT_PROF(FSHT_KCAT_ANALYSIS);
        FSHT_TRY(fsht_launch_analysis_fp64(p, 0, W0, nullptr, alm, nullptr, nmaps, c0, kc, 0, 1,
                                           p->stream));
      }
      for (int it = 0; it < niter; ++it) {
        {
          FSHT_PROF(FSHT_KCAT_SYNTHESIS);
          FSHT_TRY(fsht_launch_synthesis_fp64(p, 0, alm, nullptr, W1, nullptr, nmaps, c0, kc,
                                              p->stream));
        }
        {
          FSHT_PROF(FSHT_KCAT_RESIDUAL);
          FSHT_TRY(fsht_launch_fourier_residual(p, W0, W1, kc, method, p->stream));
        }
        {
          FSHT_PROF(FSHT_KCAT_ANALYSIS);
          FSHT_TRY(fsht_launch_analysis_fp64(p, 0, W1, nullptr, alm, nullptr, nmaps, c0, kc, 1,
                                             1, p->stream));
        }
      }
    }
    // whatever the waves did not return yet (all of it for FP64 or niter > 0)
    if (hx) FSHT_TRY(xfer_orders_done(p, *hx, alm, nmaps, 0, p->lmax + 1, c0, kc));
  }
  if (hx) FSHT_TRY(xfer_join(p));
  return FSHT_OK;
}

int fsht_t2alm(fsht_plan* p, const double* maps, double* alm, int nmaps, int niter, int method) {
  FSHT_TRY(check_call(p, nmaps, maps, alm));
  if (niter < 0 || method < 0 || method > 1) {
    fsht_set_error("niter = %d, method = %d: need niter >= 0 and method 0 (old) or 1 (new)",
                   niter, method);
    return FSHT_EINVAL;
  }
  return t2alm_impl(p, maps, alm, nmaps, niter, method, nullptr);
}

int fsht_t2alm_host(fsht_plan* p, const double* host_maps, double* host_alm, double* dev_maps,
                    double* dev_alm, int nmaps, int niter, int method) {
  FSHT_TRY(check_call(p, nmaps, dev_alm, dev_alm));
  if (!host_maps || !host_alm) {
    fsht_set_error("t2alm_host: null host buffer");
    return FSHT_EINVAL;
  }
  const double* direct =
      p->host_staged ? nullptr : host_direct(host_maps, sizeof(double) * (size_t)p->npix * nmaps);
  if (!direct && !dev_maps) {
    fsht_set_error("t2alm_host: dev_maps is null and the maps are not read in place "
                   "(not inside one fsht_host_alloc block, or staged reads requested)");
    return FSHT_EINVAL;
  }
  if (niter < 0 || method < 0 || method > 1) {
    fsht_set_error("niter = %d, method = %d: need niter >= 0 and method 0 (old) or 1 (new)",
                   niter, method);
    return FSHT_EINVAL;
  }
  if (!p->xfer) {
    fsht_set_error("t2alm_host needs a plan that owns its workspace (not FSHT_FLAG_TABLES_ONLY)");
    return FSHT_EUNSUPPORTED;
  }
  HostXfer hx;
  hx.hmaps = host_maps;
  hx.direct = direct;
  hx.halm = host_alm;
  return t2alm_impl(p, dev_maps, dev_alm, nmaps, niter, method, &hx);
}

int fsht_alm2t(fsht_plan* p, const double* alm, double* maps, int nmaps) {
  FSHT_TRY(check_call(p, nmaps, maps, alm));
  for (int c0 = 0; c0 < nmaps; c0 += p->kchunk) {
    const int kc = nmaps - c0 < p->kchunk ? nmaps - c0 : p->kchunk;
    double2* W0 = work_buf(p, 0, kc);
    if (p->precision == FSHT_PREC_SPLIT) {
      FSHT_TRY(split_synthesis(p, alm, W0, nmaps, c0, kc));
    } else {
      FSHT_PROF(FSHT_KCAT_SYNTHESIS);
      FSHT_TRY(fsht_launch_synthesis_fp64(p, 0, alm, nullptr, W0, nullptr, nmaps, c0, kc,
                                          p->stream));
    }
    {
      FSHT_PROF(FSHT_KCAT_FFT_INV);
      FSHT_TRY(fsht_launch_ring_fft_inv(p, W0, maps + (size_t)c0 * p->npix, p->npix, kc, p->stream));
    }
  }
  return FSHT_OK;
}

// ----------------------------------------------------------------- spin 2
// One chunk's spin-2 analysis of {S, D}(Q), {S, D}(U) into E/B (which: bit0 E, bit1 B),
// added when accumulate: the FP64 kernel, or the split form's tiles and waves.
static int pol_analysis(fsht_plan* p, const double2* WQ, const double2* WU, double* almE,
                        double* almB, int nmaps, int c0, int kc, int accumulate, int which,
                        bool started = false) {
  if (p->precision != FSHT_PREC_SPLIT) {
    FSHT_PROF(FSHT_KCAT_ANALYSIS);
    return fsht_launch_analysis_fp64(p, 2, WQ, WU, almE, almB, nmaps, c0, kc, accumulate, which,
                                     p->stream);
  }
  if (!p->d_poltab) {
    fsht_set_error("spin-2 split analysis needs a plan created with FSHT_FLAG_POL");
    return FSHT_EUNSUPPORTED;
  }
  // every alm element of the chunk is written by one unit of the contraction (its first pass
  // stores, later passes add), so alm needs no clearing
  if (!started) FSHT_TRY(lam_start(p, fsht_launch_split_lambda_pol));
  // Slicing of Q and U runs one wave ahead on the second auxiliary stream, as in the spin-0
  // analysis: wave w's tiles of Q and U sit in quarters 2 (w & 1) and 2 (w & 1) + 1 of d_ws /
  // d_eb (quarters 0 and 1 without the auxiliary streams).
  const bool ahead = p->aux2 != nullptr && p->aux != nullptr;
  const size_t ws1 = fsht_split_ws_bytes(p, kc);
  const size_t eb1 = fsht_split_eb_bytes(p, kc) / sizeof(int);
  auto quarter = [&](int w, int field) -> size_t {
    return (ahead ? 2 * (size_t)(w & 1) : 0) + (size_t)field;
  };
  auto slice_on = [&](int w, cudaStream_t st) -> int {
    FSHT_PROF_ON(FSHT_KCAT_SLICE, st);
    FSHT_TRY(fsht_launch_split_slice(p, w, WQ, p->d_ws + quarter(w, 0) * ws1,
                                     p->d_eb + quarter(w, 0) * eb1, kc, st));
    return fsht_launch_split_slice(p, w, WU, p->d_ws + quarter(w, 1) * ws1,
                                   p->d_eb + quarter(w, 1) * eb1, kc, st);
  };
  if (ahead) {
    FSHT_CUDA_TRY(cudaEventRecord(p->evs[0], p->stream));
    FSHT_CUDA_TRY(cudaStreamWaitEvent(p->aux2, p->evs[0], 0));
    FSHT_TRY(slice_on(0, p->aux2));
    FSHT_CUDA_TRY(cudaEventRecord(p->evs[2], p->aux2));
  }
  for (int w = 0; w < p->nwaves; ++w) {
    if (!ahead) {
      FSHT_TRY(slice_on(w, p->stream));
    } else {
      if (w + 1 < p->nwaves) {
        // the quarters of wave w + 1 were last read by the contraction of wave w - 1
        if (w >= 1)
          FSHT_CUDA_TRY(cudaStreamWaitEvent(p->aux2, p->ev[kEvDone + ((w + 1) & 1)], 0));
        FSHT_TRY(slice_on(w + 1, p->aux2));
        FSHT_CUDA_TRY(cudaEventRecord(p->evs[2 + ((w + 1) & 1)], p->aux2));
      }
      FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->evs[2 + (w & 1)], 0));
    }
    unsigned char* lb = nullptr;
    FSHT_TRY(lam_ready(p, fsht_launch_split_lambda_pol, w, &lb));
    {
      FSHT_PROF(FSHT_KCAT_ANALYSIS);
      FSHT_TRY(fsht_launch_split_gemm_pol(p, w, p->d_ws + quarter(w, 0) * ws1,
                                          p->d_eb + quarter(w, 0) * eb1,
                                          p->d_ws + quarter(w, 1) * ws1,
                                          p->d_eb + quarter(w, 1) * eb1, lb, almE, almB, nmaps,
                                          c0, kc, accumulate, which, p->stream));
    }
    FSHT_TRY(lam_done(p, fsht_launch_split_lambda_pol, w));
  }
  if (ahead) {
    FSHT_CUDA_TRY(cudaEventRecord(p->evs[1], p->aux2));
    FSHT_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->evs[1], 0));
  }
  return lam_finish(p);
}

// One chunk's spin-2 synthesis of E/B into {G_N, G_S} of Q and U: the FP64 kernel, or the
// split form's tiles and waves.
static int pol_synthesis(fsht_plan* p, const double* almE, const double* almB, double2* WQ,
                         double2* WU, int nmaps, int c0, int kc) {
  if (p->precision != FSHT_PREC_SPLIT) {
    FSHT_PROF(FSHT_KCAT_SYNTHESIS);
    return fsht_launch_synthesis_fp64(p, 2, almE, almB, WQ, WU, nmaps, c0, kc, p->stream);
  }
  if (!p->d_poltab) {
    fsht_set_error("spin-2 split synthesis needs a plan created with FSHT_FLAG_POL");
    return FSHT_EUNSUPPORTED;
  }
  unsigned char* wse = p->d_ws;
  unsigned char* wsb = p->d_ws + fsht_split_ws_bytes(p, kc);
  int* ebe = p->d_eb;
  int* ebb = p->d_eb + fsht_split_eb_bytes(p, kc) / sizeof(int);
  // the first pass of every unit stores G_N and G_S, later passes add: no clearing
  FSHT_TRY(lam_start(p, fsht_launch_split_lambdaT_pol));
  for (int w = 0; w < p->nwaves; ++w) {
    {
      FSHT_PROF(FSHT_KCAT_SLICE);
      FSHT_TRY(fsht_launch_split_slice_alm(p, w, almE, wse, ebe, nmaps, c0, kc, p->stream));
      FSHT_TRY(fsht_launch_split_slice_alm(p, w, almB, wsb, ebb, nmaps, c0, kc, p->stream));
    }
    unsigned char* lb = nullptr;
    FSHT_TRY(lam_ready(p, fsht_launch_split_lambdaT_pol, w, &lb));
    {
      FSHT_PROF(FSHT_KCAT_SYNTHESIS);
      FSHT_TRY(fsht_launch_split_synth_pol(p, w, wse, ebe, wsb, ebb, lb, WQ, WU, kc,
                                           p->stream));
    }
    FSHT_TRY(lam_done(p, fsht_launch_split_lambdaT_pol, w));
  }
  return lam_finish(p);
}

static int qu_analysis(fsht_plan* p, const double* Q, const double* U, double* almE,
                       double* almB, int nmaps, int niter, int method, int which) {
  FSHT_TRY(need_bufs(p, niter > 0 ? 4 : 2));
  for (int c0 = 0; c0 < nmaps; c0 += p->kchunk) {
    const int kc = nmaps - c0 < p->kchunk ? nmaps - c0 : p->kchunk;
    double2* WQ = work_buf(p, 0, kc);
    double2* WU = work_buf(p, 1, kc);
    const bool pre = p->precision == FSHT_PREC_SPLIT && p->d_poltab;
    if (pre) FSHT_TRY(lam_start(p, fsht_launch_split_lambda_pol));   // overlaps the FFTs
    {
      FSHT_PROF(FSHT_KCAT_FFT_FWD);
      FSHT_TRY(fsht_launch_ring_fft_fwd(p, Q + (size_t)c0 * p->npix, p->npix, kc, WQ, p->stream));
    }
    {
      FSHT_PROF(FSHT_KCAT_FFT_FWD);
      FSHT_TRY(fsht_launch_ring_fft_fwd(p, U + (size_t)c0 * p->npix, p->npix, kc, WU, p->stream));
    }
    FSHT_TRY(pol_analysis(p, WQ, WU, almE, almB, nmaps, c0, kc, 0, which, pre));
    if (niter > 0) {
      double2* RQ = work_buf(p, 2, kc);
      double2* RU = work_buf(p, 3, kc);
      for (int it = 0; it < niter; ++it) {
        FSHT_TRY(pol_synthesis(p, almE, almB, RQ, RU, nmaps, c0, kc));
        {
          FSHT_PROF(FSHT_KCAT_RESIDUAL);
          FSHT_TRY(fsht_launch_fourier_residual(p, WQ, RQ, kc, method, p->stream));
        }
        {
          FSHT_PROF(FSHT_KCAT_RESIDUAL);
          FSHT_TRY(fsht_launch_fourier_residual(p, WU, RU, kc, method, p->stream));
        }
        FSHT_TRY(pol_analysis(p, RQ, RU, almE, almB, nmaps, c0, kc, 1, which));
      }
    }
  }
  return FSHT_OK;
}

int fsht_qu2eb(fsht_plan* p, const double* Q, const double* U, double* almE, double* almB,
               int nmaps, int niter) {
  FSHT_TRY(check_call(p, nmaps, Q, U));
  if (!almE || !almB || niter < 0) {
    fsht_set_error("null alm pointer or niter < 0");
    return FSHT_EINVAL;
  }
  return qu_analysis(p, Q, U, almE, almB, nmaps, niter, 0, 3);
}

int fsht_qu2e(fsht_plan* p, const double* Q, const double* U, double* almE, int nmaps) {
  FSHT_TRY(check_call(p, nmaps, Q, U));
  if (!almE) {
    fsht_set_error("null alm pointer");
    return FSHT_EINVAL;
  }
  return qu_analysis(p, Q, U, almE, nullptr, nmaps, 0, 0, 1);
}

int fsht_qu2b(fsht_plan* p, const double* Q, const double* U, double* almB, int nmaps) {
  FSHT_TRY(check_call(p, nmaps, Q, U));
  if (!almB) {
    fsht_set_error("null alm pointer");
    return FSHT_EINVAL;
  }
  return qu_analysis(p, Q, U, nullptr, almB, nmaps, 0, 0, 2);
}

int fsht_eb2qu(fsht_plan* p, const double* almE, const double* almB, double* Q, double* U,
               int nmaps) {
  FSHT_TRY(check_call(p, nmaps, almE, almB));
  if (!Q || !U) {
    fsht_set_error("null map pointer");
    return FSHT_EINVAL;
  }
  FSHT_TRY(need_bufs(p, 2));
  for (int c0 = 0; c0 < nmaps; c0 += p->kchunk) {
    const int kc = nmaps - c0 < p->kchunk ? nmaps - c0 : p->kchunk;
    double2* WQ = work_buf(p, 0, kc);
    double2* WU = work_buf(p, 1, kc);
    FSHT_TRY(pol_synthesis(p, almE, almB, WQ, WU, nmaps, c0, kc));
    {
      FSHT_PROF(FSHT_KCAT_FFT_INV);
      FSHT_TRY(fsht_launch_ring_fft_inv(p, WQ, Q + (size_t)c0 * p->npix, p->npix, kc, p->stream));
    }
    {
      FSHT_PROF(FSHT_KCAT_FFT_INV);
      FSHT_TRY(fsht_launch_ring_fft_inv(p, WU, U + (size_t)c0 * p->npix, p->npix, kc, p->stream));
    }
  }
  return FSHT_OK;
}

}  // extern "C"
