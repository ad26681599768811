/*
 * fastsht_gb300 — C ABI of the batched HEALPix spherical-harmonic transform path
 * for NVIDIA GB300 (sm_103a).
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns an
 * int status (FSHT_OK = 0, negative on error) and never throws.  The text of the
 * last error of the calling thread is available from fsht_last_error().
 *
 * Array conventions (identical to the reference's Fortran-order NumPy arrays):
 *   maps : float64, nmaps x npix, each map contiguous (reference: maps(npix, nsim)
 *          in Fortran order), HEALPix RING ordering, npix = 12 nside^2.
 *   alm  : float64, (lmax+1) x (lmax+1) x nmaps with the map index fastest
 *          (reference: alm(nsim, 0:lmax, 0:lmax) in Fortran order), "square-real"
 *          packing: Re a_lm at [m][l][k] (l >= m), Im a_lm at [lmax+1-m][l-m][k]
 *          (m >= 1).  Slots not named by this packing do not exist: every one of
 *          the (lmax+1)^2 slots is either a Re or an Im of some a_lm.
 * Transform entry points take DEVICE pointers and run asynchronously on the
 * plan's stream (fsht_plan_set_stream).  The *_host entry points take host
 * pointers and enqueue the copies with the transform on the same stream.
 */
#ifndef FASTSHT_GB300_H
#define FASTSHT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fsht_plan fsht_plan;

enum {
  FSHT_OK = 0,
  FSHT_EINVAL = -1,       /* bad argument (sizes, null pointers, nmaps > plan) */
  FSHT_ENOMEM = -2,       /* device allocation failed                          */
  FSHT_ECUDA = -3,        /* CUDA runtime error (message in fsht_last_error)   */
  FSHT_ETIMEOUT = -4,     /* a bounded device-side wait expired                */
  FSHT_EUNSUPPORTED = -5, /* size or mode outside what this build supports     */
  FSHT_ERANGE = -6        /* split form: a value missed its digit scale (e.g. a
                             non-finite input); the results of that work are invalid */
};

enum { FSHT_PREC_FP64 = 0, FSHT_PREC_SPLIT = 1 };

/* Plan flags: which workspace buffers to hold (reference nbuff, SHT.py:52-59).
 * FSHT_FLAG_TABLES_ONLY: geometry and FFT tables without a workspace (for plans
 * that only lend their tables to a batch; transforms on them return FSHT_EINVAL). */
enum { FSHT_FLAG_POL = 1, FSHT_FLAG_ITER = 2, FSHT_FLAG_TABLES_ONLY = 4 };

/* Plan creation: replaces the reference's SHT.__init__ -> sht_data_alloc +
 * sht_set_data (SHT.py:17-62; src/sht_data_init.f90:2-269, 275-311).  Computes
 * the ring geometry, ring-skip table, FFT tables and workspace on the device.
 *   nside      power of two, 1..2048
 *   lmax       0 <= lmax <= 4*nside
 *   nmaps_max  largest nmaps a transform call on this plan will pass
 *   flags      FSHT_FLAG_POL for spin-2 (Q/U) transforms, FSHT_FLAG_ITER for
 *              niter > 0 (each doubles the workspace, like the reference's nbuff)
 *   precision  FSHT_PREC_FP64 (plain, all FP64) or FSHT_PREC_SPLIT (the Legendre
 *              contractions of t2alm, alm2t, qu2eb / qu2e / qu2b and eb2qu as BF16 slice
 *              products on the tensor cores, the ring FFTs of t2alm in df64; max relative
 *              alm error ~1e-9..3e-8 against FP64)
 *   workspace_limit_bytes  upper bound for the plan's workspace (0 = default 16 GiB,
 *              40 GiB for FSHT_PREC_SPLIT); maps are processed in chunks that fit.
 *   stream     cudaStream_t (NULL = legacy default stream) */
int fsht_plan_create(int nside, int lmax, int nmaps_max, int flags, int precision,
                     size_t workspace_limit_bytes, void* stream, fsht_plan** plan);
/* Releases a plan (reference: sht_data_free, src/sht_data_init.f90:319-372). */
int fsht_plan_destroy(fsht_plan* plan);
int fsht_plan_set_stream(fsht_plan* plan, void* stream);
/* Device bytes the plan holds (tables + workspace) and maps per chunk. */
int fsht_plan_info(const fsht_plan* plan, size_t* device_bytes, int* maps_per_chunk);
/* First kept ring i0(m) for m = 0..lmax (reference SHT_ring_skip_table/<nside>.bin,
 * read at SHT.py:31-32); out must hold lmax+1 ints (host memory). */
int fsht_plan_ring_skip(const fsht_plan* plan, int* out);

/* Temperature analysis.  niter = 0: reference t2alm (src/sht_main.f90:38-89).
 * niter > 0, method 0: t2alm_iter_old (src/sht_main.f90:276-367);
 * method 1: t2alm_iter (src/sht_main.f90:171-264). */
int fsht_t2alm(fsht_plan* plan, const double* maps, double* alm, int nmaps,
               int niter, int method);
/* fsht_t2alm from and to host memory, with the transfers overlapped with the transform.
 * Maps inside one fsht_host_alloc block (mapped into the device's address space) are read in
 * place by the forward FFT over the host link, every value once, with no staging copy (unless
 * fsht_plan_set_host_read(plan, 0)); other maps go to dev_maps in sub-batches on the plan's
 * copy stream and each is forward-transformed as soon as it lands.  alm columns go from
 * dev_alm back to host_alm as soon as they are final (after each wave of the split form when
 * niter = 0, else after the chunk).  Replaces the reference's host-side SHT.t2alm call
 * (SHT.py:72-107 over sht_main.f90:38-89, whose maps and alm live in host memory).
 * dev_maps / dev_alm: device buffers of the same layouts, provided by the caller (nothing is
 * allocated here); dev_maps may be null when the maps are read in place (fsht_host_mapped).
 * Host buffers should be pinned for the copies to run asynchronously.  Results equal
 * fsht_t2alm's; when the call returns the work is enqueued on the plan's stream
 * (fsht_plan_sync waits for it; the host buffers must stay valid until then).  Needs a plan
 * that owns its workspace. */
int fsht_t2alm_host(fsht_plan* plan, const double* host_maps, double* host_alm,
                    double* dev_maps, double* dev_alm, int nmaps, int niter, int method);
/* How fsht_t2alm_host obtains host maps: direct = 1 (the default) reads maps that lie in one
 * fsht_host_alloc block in place, direct = 0 always copies them to dev_maps first, direct = 2
 * reads them in place in chunks: in the split form (niter = 0, 128 or more maps, a workspace
 * of two chunks) the maps run in chunks of a multiple of 64, each chunk's forward FFT reading
 * the host link while the previous chunk's contraction runs on high-priority streams (on GB300
 * this measured slower than one chunk: the FFT needs most SMs to keep the link busy).  Results
 * are the same in every mode.  No counterpart in the reference. */
int fsht_plan_set_host_read(fsht_plan* plan, int direct);
/* Temperature synthesis: reference alm2t (src/sht_main.f90:96-155). */
int fsht_alm2t(fsht_plan* plan, const double* alm, double* maps, int nmaps);
/* Temperature analysis that allocates no device memory and needs no plan
 * (niter = 0, plain FP64, same results as fsht_t2alm within 1e-11 relative).
 * No counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc where they run the transform: a host application that reserved all
 * device memory for its own pool and gives plug-ins buffers but no right to
 * allocate, or a latency-critical loop where an allocation would synchronise the
 * device.  Scratch comes from one fixed 32 MiB array of device memory inside the
 * library (every GPU that loads the library holds it until exit).  A size is
 * accepted when its tables plus one map's phase matrix fit in that array: every
 * nside <= 256 at any lmax <= 4 nside, and nside 512 up to lmax 167; larger lmax
 * at nside 512, and nside 1024 and 2048, return FSHT_EUNSUPPORTED.
 * maps / alm are device pointers (layouts as above); stream is a cudaStream_t.
 * The first call on a device looks up the scratch address with that device
 * current: make it before any stream capture.  Calls share the scratch, so calls
 * that overlap on the GPU (other streams or threads) race; calls on one stream
 * are ordered. */
int fsht_t2alm_noalloc(int nside, int lmax, const double* maps, double* alm, int nmaps,
                       void* stream);

/* Spin-2 analysis.  niter = 0: QU2EB (src/sht_main.f90:383-436);
 * niter > 0: qu2eb_iter_old (src/sht_main.f90:563-673). */
int fsht_qu2eb(fsht_plan* plan, const double* Q, const double* U, double* almE,
               double* almB, int nmaps, int niter);
/* E only: QU2E (src/sht_main.f90:955-1005). */
int fsht_qu2e(fsht_plan* plan, const double* Q, const double* U, double* almE, int nmaps);
/* B only: QU2B (src/sht_main.f90:1016-1064). */
int fsht_qu2b(fsht_plan* plan, const double* Q, const double* U, double* almB, int nmaps);
/* Spin-2 synthesis: EB2QU (src/sht_main.f90:1079-1147). */
int fsht_eb2qu(fsht_plan* plan, const double* almE, const double* almB, double* Q,
               double* U, int nmaps);

/* Square-real alm -> healpy layout (interleaved re,im per (l,m), index
 * m(2 lmax+1-m)/2 + l, map index slowest: out[k][idx][2]).  Reference:
 * convert_alm_healpy1 (src/convert_alm.f90:34-56) as used by
 * SHT.convert_alm_healpy (SHT.py:204-210).  Device pointers, plan's stream. */
int fsht_convert_alm_healpy(fsht_plan* plan, const double* alm, double* alm_hp, int nmaps);
/* Inverse: convert_alm_healpy_inv1 (src/convert_alm.f90:87-107). */
int fsht_convert_alm_healpy_inv(fsht_plan* plan, const double* alm_hp, double* alm, int nmaps);

/* ---------------------------------------------------------------- alm utilities
 * Square-real alm, device pointers, layout [lmax+1][lmax+1][nmaps] (map fastest), async on
 * `stream` (a cudaStream_t, NULL = legacy default stream).  No plan needed.
 *
 * fsht_alm2cl: cl[l][k] = sum_m fac_m Re(a1_lm conj a2_lm) / (2l+1), fac_0 = 1, fac_m = 2,
 *   zero for l < lmin; alm2 = NULL or alm1 gives the auto spectrum.  cl: [lmax+1][nmaps].
 *   Replaces alm2cl_TEB1 / alm2cl_T1 (src/alm2cl_TEB.f90:22-110), one spectrum per call.
 * fsht_alm_filter: alm(l, m) *= win[l].  Replaces filt_alm1 (src/filt_alm.f90:16-37).
 * fsht_alm_norm: out = in * fac[l] + shift[l], the m = 0 entries also times m0.  Replaces
 *   norm_alm1 (src/norm_alm.f90:14-35).
 * fsht_cl2alm: Gaussian alm with spectra cl ([lmax+1][ncl], ncl = 1: TT, or 6: TT EE BB TE TB
 *   EB), zero for l < lmin, from a counter-based generator keyed by seed.  Replaces
 *   cl2alm_TEB1 / cl2alm_T1 (src/cl2alm_TEB.f90:25-171); the reference's MKL MCG31 stream is
 *   not reproduced (same statistics, different draws).  almE / almB may be NULL when ncl = 1. */
int fsht_alm2cl(const double* alm1, const double* alm2, double* cl, int lmax, int nmaps,
                int lmin, void* stream);
int fsht_alm_filter(double* alm, const double* win, int lmax, int nmaps, void* stream);
int fsht_alm_norm(const double* alm_in, double* alm_out, const double* fac, const double* shift,
                  double m0, int lmax, int nmaps, void* stream);
int fsht_cl2alm(const double* cl, int ncl, int lmin, int lmax, int nmaps, unsigned long long seed,
                double* almT, double* almE, double* almB, void* stream);

/* Per-kernel timing with CUDA events on the plan's stream (no host sync per
 * launch).  Categories: FSHT_KCAT_*.  fsht_profile_read synchronises the stream,
 * returns per-category launch counts and summed milliseconds, and clears them. */
enum {
  FSHT_KCAT_FFT_FWD = 0,
  FSHT_KCAT_FFT_INV = 1,
  FSHT_KCAT_ANALYSIS = 2,
  FSHT_KCAT_SYNTHESIS = 3,
  FSHT_KCAT_RESIDUAL = 4,
  FSHT_KCAT_SLICE = 5,      /* split form: phase matrix -> BF16 digit tiles */
  FSHT_KCAT_OTHER = 6,
  FSHT_KCAT_LAMBDA = 7,     /* split form: FP64 recursion -> BF16 lambda digit tiles */
  FSHT_KCAT_COUNT = 8
};
int fsht_profile_enable(fsht_plan* plan, int on);
int fsht_profile_read(fsht_plan* plan, int ncat, int* launches, double* total_ms);

/* Measures this device's FP64 FMA throughput (TFLOP/s) with a DFMA loop kernel:
 * the roofline denominator for the FP64 kernels. */
int fsht_measure_fp64_peak(double* tflops);
/* The same for FP32 FMAs: the roofline denominator of the split form's ring FFT, which
 * runs in df64 (FP32-pair) arithmetic. */
int fsht_measure_fp32_peak(double* tflops);
/* The same for FP64 tensor-core products (mma.sync m8n8k4 f64, DMMA), the unit the reference's
 * cuBLAS DGEMMs run on (src/sht_core.f90:51-57): on GB300 it is slower than the FP64 FMA
 * pipe, which is why the plain contraction uses DFMA.  No counterpart in the reference. */
int fsht_measure_dmma_peak(double* tflops);
/* BF16 tcgen05 UMMA throughput (TFLOP/s) of the split contraction's k-step (ten 128 x n_cols x 16
 * digit products) with its operands already in shared memory, one CTA per SM: the ceiling of
 * the contraction's tile shape (n_cols 128) and of a wider one (256).  No counterpart in the
 * reference. */
int fsht_measure_umma_rate(int n_cols, double* tflops);

/* Runs one stage of the pipeline on device buffers (testing and profiling hook;
 * no counterpart in the reference, whose stages are internal):
 *   FSHT_STAGE_FFT_FWD   maps -> phase matrix {S, D}        (in: maps, out: W)
 *   FSHT_STAGE_ANALYSIS  phase matrix -> alm (spin 0)       (in: W, out: alm)
 *   FSHT_STAGE_SYNTHESIS alm -> phase matrix {G_N, G_S}     (in: alm, out: W)
 *   FSHT_STAGE_FFT_INV   phase matrix -> maps               (in: W, out: maps)
 * W is laid out [m][ring][map][2] complex (double2), ring < 2 nside, m <= lmax,
 * for nmaps <= the plan's maps_per_chunk. */
enum { FSHT_STAGE_FFT_FWD = 0, FSHT_STAGE_ANALYSIS = 1, FSHT_STAGE_SYNTHESIS = 2,
       FSHT_STAGE_FFT_INV = 3 };
int fsht_run_stage(fsht_plan* plan, int stage, const void* in, void* out, int nmaps);

/* ---------------------------------------------------------------------------
 * Batched form: many map sets with different nside / lmax / nmaps / spin /
 * precision run as one CUDA-graph launch.  No counterpart in the reference, which
 * runs one SHT instance (module-global state) and one transform per Python call
 * (SHT.py:16-227).  Buffers are device pointers fixed at creation: rerunning the
 * batch reuses them (write new inputs in place, then fsht_batch_run again).
 *   kind  T2ALM: in0 maps -> out0 alm      ALM2T: in0 alm -> out0 maps
 *         QU2EB: in0 Q, in1 U -> out0 E, out1 B
 *         EB2QU: in0 E, in1 B -> out0 Q, out1 U
 * Layouts as for the single-plan entry points, per job. */
enum { FSHT_JOB_T2ALM = 0, FSHT_JOB_ALM2T = 1, FSHT_JOB_QU2EB = 2, FSHT_JOB_EB2QU = 3 };
typedef struct fsht_job {
  int nside, lmax, nmaps, kind, precision;
  const double* in0;
  const double* in1;
  double* out0;
  double* out1;
} fsht_job;
typedef struct fsht_batch fsht_batch;
/* One table-only plan per distinct (nside, lmax, precision); workspace_budget_bytes
 * (0 = 64 GiB) is cut into nslots stream slots (0 = 4) that run jobs concurrently,
 * longest first.  autotune != 0 picks each plan's ring-FFT launch shape by timing
 * (fsht_plan_autotune).  The first fsht_batch_run captures the whole batch into a
 * CUDA graph on `stream` (NULL: a stream the batch creates; graphs cannot be captured
 * on the legacy default stream); every run (including the first) is one graph launch.
 * fsht_batch_sync waits for it. */
int fsht_batch_create(const fsht_job* jobs, int njobs, int nslots, size_t workspace_budget_bytes,
                      int autotune, void* stream, fsht_batch** batch);
int fsht_batch_run(fsht_batch* batch);
/* Number of distinct plans and of nodes in the captured graph (0 before the first run). */
int fsht_batch_info(const fsht_batch* batch, int* nplans, int* nnodes);
/* The i-th plan of a batch (0 <= i < nplans): its nside, lmax, precision and the launch shapes
 * it runs with (after autotuning, when the batch was created with it): shapes[0..4] = FFT maps
 * per CTA (0: sized from the maps of each call), FFT threads (0: the per-segment default),
 * FP64 analysis maps per CTA, FP64 rings per chunk, split ring-part k-steps (0: the kernel's
 * default).  No counterpart in the reference. */
int fsht_batch_plan_tuning(const fsht_batch* batch, int i, int* nside, int* lmax, int* precision,
                           int* shapes);
int fsht_batch_sync(fsht_batch* batch);
int fsht_batch_destroy(fsht_batch* batch);

/* One job on a caller-provided workspace and stream, using the tables of a plan
 * with the same nside / lmax / precision (typically FSHT_FLAG_TABLES_ONLY).  Jobs
 * sharing one plan may run concurrently on different streams with different
 * workspaces: this is the execution primitive of the serving loop
 * (fastsht_gb300.serve).  fsht_job_workspace gives the bytes needed for a given
 * number of maps per chunk (>= 1); a larger workspace lets more maps share a pass. */
int fsht_job_workspace(const fsht_plan* tables, const fsht_job* job, int maps_per_chunk,
                       size_t* bytes);
int fsht_run_job(const fsht_plan* tables, const fsht_job* job, void* workspace,
                 size_t workspace_bytes, void* stream);

/* Autotuner: times the ring-FFT launch shapes (maps per CTA 1..16; 256 or 512 threads, or
 * 0 = the per-segment default) on sample_maps maps and keeps the fastest in the plan, then the
 * contraction's tile shapes (fsht_plan_set_contraction); results are cached per (nside, lmax
 * bucket of 256, sample_maps, precision) for the process.  No counterpart in the reference. */
int fsht_plan_autotune(fsht_plan* plan, int sample_maps);
int fsht_plan_tuning(const fsht_plan* plan, int* maps_per_block, int* threads);
/* Contraction tile shapes (0 = the default): the FP64 analysis kernel's maps per CTA (32 or
 * 64) and rings per chunk (8, 16 or 32 for spin 0; 8 or 16 for spin 2), and the split GEMMs'
 * ring-part length in k-steps of 16 rings (16, 32 or 64; 64 keeps the exact levels' sums below
 * 2^24).  fsht_plan_autotune times the candidates on sample_maps maps after the FFT shape and
 * keeps the fastest, cached per (nside, lmax bucket of 256, sample_maps, precision); the
 * setter fixes them by hand.  Every shape gives the same transform (the FP64 sums in another
 * order, the split form's exact levels unchanged).  No counterpart in the reference, whose
 * contraction is one cuBLAS DGEMM per m (src/sht_core.f90:30-89). */
int fsht_plan_set_contraction(fsht_plan* plan, int maps_per_cta, int rings_per_chunk,
                              int part_steps);
int fsht_plan_contraction(const fsht_plan* plan, int* maps_per_cta, int* rings_per_chunk,
                          int* part_steps);

/* Blocks until the plan's stream is idle; returns FSHT_ECUDA on an async error,
 * FSHT_ETIMEOUT when a bounded device-side wait (split-precision kernels) expired since
 * the last check, and FSHT_ERANGE when a split-form kernel met a value outside its digit
 * scale (a non-finite input) since the last check (the error word is then cleared). */
int fsht_plan_sync(fsht_plan* plan);
/* The error-word check of fsht_plan_sync without synchronising any stream: call it after
 * the work of interest is known to be complete (an event, fsht_batch_sync).  No
 * counterpart in the reference. */
int fsht_plan_check(fsht_plan* plan);
/* Failure-detection self-test: enqueues on the plan's stream one bounded device-side wait
 * that nothing satisfies; the wait expires (about a second), the plan's error word is
 * raised, and the next fsht_plan_sync returns FSHT_ETIMEOUT.  No counterpart in the
 * reference. */
int fsht_selftest_wait_timeout(fsht_plan* plan);

/* Page-locked host memory (cudaHostAlloc, portable to every device and mapped into their
 * address spaces) for host buffers of fsht_t2alm_host and the SHT class's NumPy outputs: the
 * copies run asynchronously at the host link's rate, and maps in such a block are read in
 * place by fsht_t2alm_host.  No counterpart in the reference. */
int fsht_host_alloc(size_t bytes, void** ptr);
int fsht_host_free(void* ptr);
/* *mapped = 1 when host bytes [ptr, ptr + bytes) lie inside one fsht_host_alloc block that
 * the current device can read in place (fsht_t2alm_host then needs no dev_maps), else 0. */
int fsht_host_mapped(const void* ptr, size_t bytes, int* mapped);

/* Copies the calling thread's last error message into buf (NUL-terminated);
 * returns its full length. */
int fsht_last_error(char* buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* FASTSHT_GB300_H */
