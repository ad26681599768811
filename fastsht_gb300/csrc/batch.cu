// Batched form: many map sets of different nside / lmax / nmaps / spin / precision
// executed as one CUDA-graph launch, plus the autotuner that picks the ring-FFT
// launch shape and the contraction's tile shapes per (nside, lmax) bucket.
//
// The reference runs one SHT instance per process and one transform at a time
// (module-global state, SHT.py:16-62); there it takes one Python call per map set.
// Here a batch owns one table-only plan per distinct (nside, lmax, precision), a
// fixed workspace budget cut into stream slots, and a CUDA graph captured on the
// first run: every later run is a single cudaGraphLaunch over all jobs, with
// independent jobs overlapping on the GPU through the slots' streams.
#include "common.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

struct fsht_batch {
  std::vector<fsht_job> jobs;
  std::vector<fsht_plan*> plans;   // owned, one per key
  std::vector<int> job_plan;
  std::vector<int> order;          // launch order (largest first)
  int nslots = 0;
  std::vector<cudaStream_t> slot_streams;
  std::vector<unsigned char*> arenas;
  size_t arena_bytes = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;         // created here when the caller passed the legacy stream
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<cudaEvent_t> events;
};

namespace {

constexpr size_t kDefaultBatchBudget = 64ull << 30;

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Workspace a job needs for kc maps per chunk, laid out as [W buffers][WS][EB].
struct JobLayout {
  int kc, nbuf;
  size_t w_bytes, ws_off, eb_off, lb_off, total;
};

JobLayout job_layout(const fsht_plan* p, const fsht_job& j, int kc) {
  JobLayout L;
  L.kc = kc;
  const bool pol = j.kind == FSHT_JOB_QU2EB || j.kind == FSHT_JOB_EB2QU;
  L.nbuf = pol ? 2 : 1;
  const size_t per_map = (size_t)(p->lmax + 1) * p->nnorth * 2 * sizeof(double2);
  L.w_bytes = per_map * L.nbuf * kc;
  L.ws_off = align_up(L.w_bytes);
  L.eb_off = L.ws_off;
  L.lb_off = L.ws_off;
  L.total = L.ws_off;
  if (p->precision == FSHT_PREC_SPLIT) {
    const bool pol2 = j.kind == FSHT_JOB_QU2EB || j.kind == FSHT_JOB_EB2QU;
    const size_t f = pol2 ? 2 : 1;   // spin 2: tiles of Q and U (or E and B)
    L.eb_off = align_up(L.ws_off + f * fsht_split_ws_bytes(p, kc));
    L.lb_off = align_up(L.eb_off + f * fsht_split_eb_bytes(p, kc));
    L.total = align_up(L.lb_off + p->lbuf_bytes);
  }
  return L;
}

double job_cost(const fsht_job& j) {
  const double f = 4.0 * j.nside * (j.lmax + 1.0) * (j.lmax + 2.0) * j.nmaps;
  const bool pol = j.kind == FSHT_JOB_QU2EB || j.kind == FSHT_JOB_EB2QU;
  return pol ? 4 * f : f;
}

int run_job(const fsht_plan* base, const fsht_job& j, unsigned char* arena, size_t arena_bytes,
            cudaStream_t s) {
  int kc = j.nmaps;
  while (kc > 1 && job_layout(base, j, kc).total > arena_bytes) --kc;
  const JobLayout L = job_layout(base, j, kc);
  if (L.total > arena_bytes) {
    fsht_set_error("batch job (nside %d, lmax %d) needs %zu bytes of workspace per slot, above "
                   "the slot's %zu", j.nside, j.lmax, L.total, arena_bytes);
    return FSHT_ENOMEM;
  }
  fsht_plan jp = *base;          // shallow view: shared tables, this slot's stream/workspace
  jp.stream = s;
  jp.nmaps_max = j.nmaps;
  jp.kchunk = kc;
  jp.nbuf = L.nbuf;
  jp.d_work = reinterpret_cast<double2*>(arena);
  jp.work_bytes = L.w_bytes;
  jp.d_ws = arena + L.ws_off;
  jp.d_eb = reinterpret_cast<int*>(arena + L.eb_off);
  jp.d_lbuf = arena + L.lb_off;
  jp.prof = nullptr;
  switch (j.kind) {
    case FSHT_JOB_T2ALM: return fsht_t2alm(&jp, j.in0, j.out0, j.nmaps, 0, 0);
    case FSHT_JOB_ALM2T: return fsht_alm2t(&jp, j.in0, j.out0, j.nmaps);
    case FSHT_JOB_QU2EB: return fsht_qu2eb(&jp, j.in0, j.in1, j.out0, j.out1, j.nmaps, 0);
    case FSHT_JOB_EB2QU: return fsht_eb2qu(&jp, j.in0, j.in1, j.out0, j.out1, j.nmaps);
    default:
      fsht_set_error("unknown job kind %d", j.kind);
      return FSHT_EINVAL;
  }
}

// ------------------------------------------------------------------ autotuner
std::mutex g_tune_mu;
// (nside, lmax bucket, maps, df64 FFT) -> (maps per CTA, threads; 0 = per-segment default)
std::map<std::tuple<int, int, int, int>, std::pair<int, int>> g_tune;
// (nside, lmax bucket, maps, precision) -> contraction tile shape (ana_mt, ana_rc, split_part)
std::map<std::tuple<int, int, int, int>, std::tuple<int, int, int>> g_tune_c;

// Times one T analysis of the sample maps per candidate contraction tile shape and keeps the
// fastest in the plan.  The ring FFT is the same for every candidate, so the fastest call has
// the fastest contraction.  Plans that own a workspace run it there; table-only plans through a
// job view on a temporary arena.
int tune_contraction(fsht_plan* p, const double* maps, int sample_maps) {
  struct Cand {
    int mt, rc, part;
  };
  std::vector<Cand> cands;
  if (p->precision == FSHT_PREC_SPLIT) {
    for (int part : {64, 32, 16}) cands.push_back({0, 0, part});
  } else {
    for (int mt : {64, 32})
      for (int rc : {16, 32, 8}) cands.push_back({mt, rc, 0});
  }
  const size_t L1 = (size_t)p->lmax + 1;
  fsht_job j{};
  j.nside = p->nside;
  j.lmax = p->lmax;
  j.nmaps = sample_maps;
  j.kind = FSHT_JOB_T2ALM;
  j.precision = p->precision;
  j.in0 = maps;
  double* alm = nullptr;
  unsigned char* arena = nullptr;
  size_t arena_bytes = 0;
  FSHT_CUDA_TRY(cudaMalloc(&alm, sizeof(double) * L1 * L1 * sample_maps));
  j.out0 = alm;
  const bool own = p->d_work != nullptr && sample_maps <= p->kchunk;
  int rc = FSHT_OK;
  if (!own) {
    arena_bytes = job_layout(p, j, sample_maps).total;
    cudaError_t e = cudaMalloc(&arena, arena_bytes);
    if (e != cudaSuccess) {
      cudaFree(alm);
      fsht_set_error("autotune: cudaMalloc(%zu): %s", arena_bytes, cudaGetErrorString(e));
      return FSHT_ENOMEM;
    }
  }
  auto run = [&]() -> int {
    return own ? fsht_t2alm(p, maps, alm, sample_maps, 0, 0)
               : run_job(p, j, arena, arena_bytes, p->stream);
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float best = 1e30f;
  Cand pick = cands[0];
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = FSHT_ECUDA;
  for (size_t c = 0; c < cands.size() && !rc; ++c) {
    p->ana_mt = cands[c].mt;
    p->ana_rc = cands[c].rc;
    p->split_part = cands[c].part;
    if ((rc = run())) break;   // warm-up (kernel loading)
    cudaEventRecord(e0, p->stream);
    for (int r = 0; r < 2 && !rc; ++r) rc = run();
    cudaEventRecord(e1, p->stream);
    if (rc) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = FSHT_ECUDA;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      pick = cands[c];
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(alm);
  if (arena) cudaFree(arena);
  p->ana_mt = pick.mt;
  p->ana_rc = pick.rc;
  p->split_part = pick.part;
  return rc ? rc : fsht_plan_check(p);
}

}  // namespace

extern "C" int fsht_plan_autotune(fsht_plan* p, int sample_maps) {
  if (!p) {
    fsht_set_error("null plan");
    return FSHT_EINVAL;
  }
  if (sample_maps < 1) sample_maps = 1;
  const auto key = std::make_tuple(p->nside, (p->lmax + 255) / 256, sample_maps,
                                   p->d_tw_df ? 1 : 0);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    auto itc = g_tune_c.find(std::make_tuple(p->nside, (p->lmax + 255) / 256, sample_maps,
                                             p->precision));
    if (it != g_tune.end() && itc != g_tune_c.end()) {
      p->fft_mpb = it->second.first;
      p->fft_threads = it->second.second;
      std::tie(p->ana_mt, p->ana_rc, p->split_part) = itc->second;
      return FSHT_OK;
    }
  }
  if (p->d_work && sample_maps > p->kchunk && p->kchunk > 0) sample_maps = p->kchunk;
  double* maps = nullptr;
  double2* W = p->d_work;
  double2* W_tmp = nullptr;
  if (!W) {
    FSHT_CUDA_TRY(cudaMalloc(&W_tmp, sizeof(double2) * 2 * (size_t)(p->lmax + 1) * p->nnorth *
                                         sample_maps));
    W = W_tmp;
  }
  FSHT_CUDA_TRY(cudaMalloc(&maps, sizeof(double) * p->npix * sample_maps));
  FSHT_CUDA_TRY(cudaMemsetAsync(maps, 0, sizeof(double) * p->npix * sample_maps, p->stream));
  cudaEvent_t e0, e1;
  FSHT_CUDA_TRY(cudaEventCreate(&e0));
  FSHT_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_mpb = 0, best_thr = 0;
  const int mpbs[] = {1, 2, 4, 8, 16};
  const int thrs[] = {256, 512, 0};
  int rc = FSHT_OK;
  for (int thr : thrs) {
    for (int mpb : mpbs) {
      if (mpb > sample_maps && mpb != 1) continue;
      p->fft_mpb = mpb;
      p->fft_threads = thr;
      if ((rc = fsht_launch_ring_fft_fwd(p, maps, p->npix, sample_maps, W, p->stream))) break;
      cudaEventRecord(e0, p->stream);
      for (int r = 0; r < 3 && !rc; ++r)
        rc = fsht_launch_ring_fft_fwd(p, maps, p->npix, sample_maps, W, p->stream);
      cudaEventRecord(e1, p->stream);
      if (rc) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = FSHT_ECUDA;
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        best_mpb = mpb;
        best_thr = thr;
      }
    }
    if (rc) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (W_tmp) cudaFree(W_tmp);
  p->fft_mpb = best_mpb;
  p->fft_threads = best_thr;
  if (!rc) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = std::make_pair(best_mpb, best_thr);
  }
  // the contraction's tile shapes, with the chosen FFT shape in place
  const auto ckey = std::make_tuple(p->nside, (p->lmax + 255) / 256, sample_maps, p->precision);
  bool cached = false;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_c.find(ckey);
    if (it != g_tune_c.end()) {
      std::tie(p->ana_mt, p->ana_rc, p->split_part) = it->second;
      cached = true;
    }
  }
  if (!rc && !cached) {
    rc = tune_contraction(p, maps, sample_maps);
    if (!rc) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune_c[ckey] = std::make_tuple(p->ana_mt, p->ana_rc, p->split_part);
    }
  }
  cudaFree(maps);
  return rc;
}

extern "C" int fsht_plan_set_contraction(fsht_plan* p, int maps_per_cta, int rings_per_chunk,
                                         int part_steps) {
  if (!p) {
    fsht_set_error("null plan");
    return FSHT_EINVAL;
  }
  if ((maps_per_cta != 0 && maps_per_cta != 32 && maps_per_cta != 64) ||
      (rings_per_chunk != 0 && rings_per_chunk != 8 && rings_per_chunk != 16 &&
       rings_per_chunk != 32) ||
      (part_steps != 0 && part_steps != 16 && part_steps != 32 && part_steps != 64)) {
    fsht_set_error("contraction shape (%d, %d, %d): need maps_per_cta 0|32|64, rings_per_chunk "
                   "0|8|16|32, part_steps 0|16|32|64", maps_per_cta, rings_per_chunk, part_steps);
    return FSHT_EINVAL;
  }
  p->ana_mt = maps_per_cta;
  p->ana_rc = rings_per_chunk;
  p->split_part = part_steps;
  return FSHT_OK;
}

extern "C" int fsht_plan_contraction(const fsht_plan* p, int* maps_per_cta, int* rings_per_chunk,
                                     int* part_steps) {
  if (!p) {
    fsht_set_error("null plan");
    return FSHT_EINVAL;
  }
  if (maps_per_cta) *maps_per_cta = p->ana_mt;
  if (rings_per_chunk) *rings_per_chunk = p->ana_rc;
  if (part_steps) *part_steps = p->split_part;
  return FSHT_OK;
}

extern "C" int fsht_plan_tuning(const fsht_plan* p, int* maps_per_block, int* threads) {
  if (!p) {
    fsht_set_error("null plan");
    return FSHT_EINVAL;
  }
  if (maps_per_block) *maps_per_block = p->fft_mpb;
  if (threads) *threads = p->fft_threads;
  return FSHT_OK;
}

// ------------------------------------------------------------------ single job
extern "C" int fsht_job_workspace(const fsht_plan* tables, const fsht_job* job, int maps_per_chunk,
                                  size_t* bytes) {
  if (!tables || !job || !bytes || maps_per_chunk < 1) {
    fsht_set_error("job_workspace: bad arguments");
    return FSHT_EINVAL;
  }
  if (job->nside != tables->nside || job->lmax != tables->lmax ||
      job->precision != tables->precision) {
    fsht_set_error("job (nside %d, lmax %d, precision %d) does not match the plan's tables",
                   job->nside, job->lmax, job->precision);
    return FSHT_EINVAL;
  }
  *bytes = job_layout(tables, *job, maps_per_chunk).total;
  return FSHT_OK;
}

extern "C" int fsht_run_job(const fsht_plan* tables, const fsht_job* job, void* workspace,
                            size_t workspace_bytes, void* stream) {
  if (!tables || !job || !workspace) {
    fsht_set_error("run_job: bad arguments");
    return FSHT_EINVAL;
  }
  if (job->nside != tables->nside || job->lmax != tables->lmax ||
      job->precision != tables->precision) {
    fsht_set_error("job (nside %d, lmax %d, precision %d) does not match the plan's tables",
                   job->nside, job->lmax, job->precision);
    return FSHT_EINVAL;
  }
  return run_job(tables, *job, static_cast<unsigned char*>(workspace), workspace_bytes,
                 (cudaStream_t)stream);
}

// ------------------------------------------------------------------ batch
extern "C" int fsht_batch_create(const fsht_job* jobs, int njobs, int nslots,
                                 size_t workspace_budget_bytes, int autotune, void* stream,
                                 fsht_batch** out) {
  if (!out || !jobs || njobs < 1) {
    fsht_set_error("batch_create: need jobs and an output pointer");
    return FSHT_EINVAL;
  }
  *out = nullptr;
  if (nslots < 1) nslots = 4;
  fsht_batch* b = new (std::nothrow) fsht_batch();
  if (!b) {
    fsht_set_error("host allocation failed");
    return FSHT_ENOMEM;
  }
  auto fail = [&](int rc) {
    fsht_batch_destroy(b);
    return rc;
  };
  b->stream = (cudaStream_t)stream;
  if (!b->stream) {   // graphs cannot be captured on the legacy default stream
    FSHT_CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->own_stream = true;
  }
  b->jobs.assign(jobs, jobs + njobs);
  std::map<std::tuple<int, int, int>, int> key_plan;
  for (int i = 0; i < njobs; ++i) {
    const fsht_job& j = jobs[i];
    if (!j.in0 || !j.out0 || j.nmaps < 1 ||
        ((j.kind == FSHT_JOB_QU2EB || j.kind == FSHT_JOB_EB2QU) && (!j.in1 || !j.out1))) {
      fsht_set_error("batch job %d: null buffer or nmaps < 1", i);
      return fail(FSHT_EINVAL);
    }
    const auto key = std::make_tuple(j.nside, j.lmax, j.precision);
    auto it = key_plan.find(key);
    if (it == key_plan.end()) {
      fsht_plan* p = nullptr;
      // tables only (spin-2 tables too in the split form); the slots hold the workspaces
      const int flags = FSHT_FLAG_TABLES_ONLY | (j.precision == FSHT_PREC_SPLIT ? FSHT_FLAG_POL : 0);
      int rc = fsht_plan_create(j.nside, j.lmax, 1, flags, j.precision, 0, b->stream, &p);
      if (rc) return fail(rc);
      b->plans.push_back(p);
      it = key_plan.emplace(key, (int)b->plans.size() - 1).first;
    }
    b->job_plan.push_back(it->second);
  }
  if (autotune) {
    // each plan tuned at the map count of its largest job (at most one 64-map tile)
    for (size_t pi = 0; pi < b->plans.size(); ++pi) {
      int sm = 1;
      for (int i = 0; i < njobs; ++i)
        if (b->job_plan[i] == (int)pi) sm = std::max(sm, std::min(jobs[i].nmaps, 64));
      int rc = fsht_plan_autotune(b->plans[pi], sm);
      if (rc) return fail(rc);
    }
  }
  b->nslots = nslots;
  const size_t budget = workspace_budget_bytes ? workspace_budget_bytes : kDefaultBatchBudget;
  b->arena_bytes = budget / nslots & ~(size_t)255;
  for (int s = 0; s < nslots; ++s) {
    cudaStream_t st;
    FSHT_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    b->slot_streams.push_back(st);
    unsigned char* a = nullptr;
    cudaError_t e = cudaMalloc(&a, b->arena_bytes);
    if (e != cudaSuccess) {
      fsht_set_error("batch workspace: cudaMalloc(%zu): %s", b->arena_bytes, cudaGetErrorString(e));
      return fail(e == cudaErrorMemoryAllocation ? FSHT_ENOMEM : FSHT_ECUDA);
    }
    b->arenas.push_back(a);
  }
  for (int i = 0; i < 2 * nslots + 1; ++i) {
    cudaEvent_t ev;
    FSHT_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    b->events.push_back(ev);
  }
  b->order.resize(njobs);
  for (int i = 0; i < njobs; ++i) b->order[i] = i;
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int x, int y) { return job_cost(jobs[x]) > job_cost(jobs[y]); });
  *out = b;
  return FSHT_OK;
}

extern "C" int fsht_batch_run(fsht_batch* b) {
  if (!b) {
    fsht_set_error("null batch");
    return FSHT_EINVAL;
  }
  if (!b->exec) {
    // capture: fork the slots off the caller's stream, greedy longest-job-first
    // assignment to the least-loaded slot, join back
    FSHT_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    int rc = FSHT_OK;
    cudaEventRecord(b->events[0], b->stream);
    for (int s = 0; s < b->nslots; ++s) cudaStreamWaitEvent(b->slot_streams[s], b->events[0], 0);
    std::vector<double> load(b->nslots, 0.0);
    for (int idx : b->order) {
      const int s = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      load[s] += job_cost(b->jobs[idx]);
      rc = run_job(b->plans[b->job_plan[idx]], b->jobs[idx], b->arenas[s], b->arena_bytes,
                   b->slot_streams[s]);
      if (rc) break;
    }
    for (int s = 0; s < b->nslots; ++s) {
      cudaEventRecord(b->events[1 + s], b->slot_streams[s]);
      cudaStreamWaitEvent(b->stream, b->events[1 + s], 0);
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) {
      fsht_set_error("batch capture: %s", cudaGetErrorString(e));
      return FSHT_ECUDA;
    }
    b->graph = g;
    FSHT_CUDA_TRY(cudaGraphInstantiate(&b->exec, g, 0));
  }
  FSHT_CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
  return FSHT_OK;
}

extern "C" int fsht_batch_info(const fsht_batch* b, int* nplans, int* nnodes) {
  if (!b) {
    fsht_set_error("null batch");
    return FSHT_EINVAL;
  }
  if (nplans) *nplans = (int)b->plans.size();
  if (nnodes) {
    size_t n = 0;
    if (b->graph) cudaGraphGetNodes(b->graph, nullptr, &n);
    *nnodes = (int)n;
  }
  return FSHT_OK;
}

extern "C" int fsht_batch_plan_tuning(const fsht_batch* b, int i, int* nside, int* lmax,
                                      int* precision, int* shapes) {
  if (!b || i < 0 || i >= (int)b->plans.size()) {
    fsht_set_error("batch_plan_tuning: no plan %d", i);
    return FSHT_EINVAL;
  }
  const fsht_plan* p = b->plans[i];
  if (nside) *nside = p->nside;
  if (lmax) *lmax = p->lmax;
  if (precision) *precision = p->precision;
  if (shapes) {
    shapes[0] = p->fft_mpb;
    shapes[1] = p->fft_threads;
    shapes[2] = p->ana_mt;
    shapes[3] = p->ana_rc;
    shapes[4] = p->split_part;
  }
  return FSHT_OK;
}

extern "C" int fsht_batch_sync(fsht_batch* b) {
  if (!b) {
    fsht_set_error("null batch");
    return FSHT_EINVAL;
  }
  FSHT_CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (fsht_plan* p : b->plans) FSHT_TRY(fsht_plan_check(p));   // expired device-side waits
  return FSHT_OK;
}

extern "C" int fsht_batch_destroy(fsht_batch* b) {
  if (!b) return FSHT_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto s : b->slot_streams) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  for (auto a : b->arenas) cudaFree(a);
  for (auto e : b->events) cudaEventDestroy(e);
  for (auto p : b->plans) fsht_plan_destroy(p);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  delete b;
  return FSHT_OK;
}
