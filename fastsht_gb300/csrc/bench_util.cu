// Measurement helpers: FP64 and FP32 FMA and FP64 tensor-core (DMMA) throughput of the current
// device, the roofline denominators of the plain-FP64 kernels and of the df64 ring FFT.
#include "common.cuh"

namespace {
__global__ void k_dfma_loop(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

extern "C" int fsht_measure_fp64_peak(double* tflops) {
  if (!tflops) {
    fsht_set_error("null output");
    return FSHT_EINVAL;
  }
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = nsm * 8, threads = 256, iters = 8000;
  double* out = nullptr;
  FSHT_CUDA_TRY(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  FSHT_CUDA_TRY(cudaEventCreate(&e0));
  FSHT_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    FSHT_CUDA_TRY(cudaEventRecord(e0, 0));
    k_dfma_loop<<<blocks, threads>>>(out, iters, 0.999, 1e-3);
    FSHT_LAUNCH_CHECK();
    FSHT_CUDA_TRY(cudaEventRecord(e1, 0));
    FSHT_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    FSHT_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *tflops = 2.0 * 8 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
  return FSHT_OK;
}

// FP32 FMA throughput (TFLOP/s): the roofline denominator of the df64 kernels, which run on
// the FP32 pipe.
namespace {
__global__ void k_ffma_loop(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

extern "C" int fsht_measure_fp32_peak(double* tflops) {
  if (!tflops) {
    fsht_set_error("null output");
    return FSHT_EINVAL;
  }
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = nsm * 8, threads = 256, iters = 40000;
  float* out = nullptr;
  FSHT_CUDA_TRY(cudaMalloc(&out, sizeof(float) * blocks * threads));
  cudaEvent_t e0, e1;
  FSHT_CUDA_TRY(cudaEventCreate(&e0));
  FSHT_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    FSHT_CUDA_TRY(cudaEventRecord(e0, 0));
    k_ffma_loop<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
    FSHT_LAUNCH_CHECK();
    FSHT_CUDA_TRY(cudaEventRecord(e1, 0));
    FSHT_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    FSHT_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *tflops = 2.0 * 8 * (double)iters * blocks * threads / (best * 1e-3) / 1e12;
  return FSHT_OK;
}

// FP64 tensor-core (DMMA) throughput (TFLOP/s): a loop of mma.sync.m8n8k4 FP64 products with
// four independent accumulators per warp.  The plain path's contraction is written for the
// FP64 FMA pipe because this figure is below fsht_measure_fp64_peak's on GB300; measuring both
// in every run keeps that choice checkable.
namespace {
__global__ void k_dmma_loop(double* out, int iters, double a, double b) {
  double acc[4][2];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    acc[j][0] = threadIdx.x + j;
    acc[j][1] = threadIdx.x - j;
  }
  const double fa = a + 1e-9 * threadIdx.x, fb = b;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile(
          "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
          : "+d"(acc[j][0]), "+d"(acc[j][1])
          : "d"(fa), "d"(fb));
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 4; ++j) s += acc[j][0] + acc[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int fsht_measure_dmma_peak(double* tflops) {
  if (!tflops) {
    fsht_set_error("null output");
    return FSHT_EINVAL;
  }
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = nsm * 8, threads = 256, iters = 2000;
  double* out = nullptr;
  FSHT_CUDA_TRY(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  FSHT_CUDA_TRY(cudaEventCreate(&e0));
  FSHT_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    FSHT_CUDA_TRY(cudaEventRecord(e0, 0));
    k_dmma_loop<<<blocks, threads>>>(out, iters, 1.0 - 1e-6, 1e-3);
    FSHT_LAUNCH_CHECK();
    FSHT_CUDA_TRY(cudaEventRecord(e1, 0));
    FSHT_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    FSHT_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  // one m8n8k4 product per warp = 8 * 8 * 4 FMAs = 512 flop
  const double warps = (double)blocks * threads / 32.0;
  *tflops = 512.0 * 4 * (double)iters * warps / (best * 1e-3) / 1e12;
  return FSHT_OK;
}

// ---------------------------------------------------------------- wait self-test
// One thread waits, with the kernels' bounded mbarrier wait, on a barrier that nothing
// arrives on: the wait gives up after its iteration limit (about a second), and the
// kernel raises the plan's error word exactly as an expired wait in the split-precision
// kernels does.  No fault, no trap, no unbounded loop.
#include "tcgen05.cuh"

namespace {
__global__ void k_wait_selftest(int* err) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    abort_flag = 0;
    tc::mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!tc::mbar_wait(&bar, 0, &abort_flag)) atomicOr(err, tc::kErrTimeout);
    tc::mbar_arrive(&bar);   // leave the barrier completed before the CTA exits
  }
}
}  // namespace

extern "C" int fsht_selftest_wait_timeout(fsht_plan* p) {
  if (!p) {
    fsht_set_error("null plan");
    return FSHT_EINVAL;
  }
  k_wait_selftest<<<1, 32, 0, p->stream>>>(p->d_err);
  FSHT_LAUNCH_CHECK();
  return FSHT_OK;
}

// ---------------------------------------------------------------- UMMA issue rate
// BF16 tcgen05 throughput (TFLOP/s) of the split contraction's k-step with operands already in
// shared memory: one CTA per SM, one thread issuing ten 128 x N x 16 UMMAs per k-step (the
// level-ordered digit products of the analysis GEMM, A digit tiles of 128 rows, B digit tiles
// of N rows) into 512 / N accumulators of N columns, no loads, no epilogue.  N = 128 is the
// contraction's tile; N = 256 shows what a wider tile would allow.  Operand tiles are zero
// (the values do not change the rate).
namespace {
constexpr int kUmmaProbeSmem = 120 * 1024;   // keeps one CTA per SM (TMEM is allocated whole)

template <int N>
__global__ void __launch_bounds__(128, 1) k_umma_loop(int iters, int* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar, step_bar;
  __shared__ uint32_t tmem_s;
  __shared__ int abort_flag;
  constexpr uint32_t kA = 128 * 32, kB = N * 32;   // one K = 16 digit tile, K-major
  for (int i = threadIdx.x; i < (int)(4 * kA + 4 * kB) / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_init(&step_bar, 1);
    abort_flag = 0;
    tc::mbar_fence_init();
  }
  if (threadIdx.x < 32) tc::tmem_alloc(&tmem_s, 512);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // zeros visible to the UMMAs
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_s;
  if (threadIdx.x == 0) {
    const uint32_t idesc = tc::umma_idesc_bf16(128, N);
    const uint32_t s_a = tc::smem_u32(smem), s_b = s_a + 4 * kA;
    constexpr int nacc = 512 / N;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
      for (int lev = 0; lev <= 3; ++lev)
#pragma unroll
        for (int aa = 0; aa <= lev; ++aa)
          tc::umma_bf16(tmem + (lev % nacc) * N, tc::umma_desc(s_a + aa * kA, 128, 256),
                        tc::umma_desc(s_b + (lev - aa) * kB, 128, 256), idesc,
                        (it > 0 || aa > 0) ? 1u : 0u);
      tc::umma_commit(&step_bar);   // as the contraction releases a ring stage per k-step
    }
    tc::umma_commit(&bar);
    if (!tc::mbar_wait(&bar, 0, &abort_flag)) atomicOr(err, tc::kErrTimeout);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(tmem, 512);
}

template <int N>
int umma_rate(int nsm, int* d_err, double* tflops) {
  FSHT_TRY(fsht_smem_limit((const void*)k_umma_loop<N>, (size_t)kUmmaProbeSmem));
  const int iters = 20000;
  cudaEvent_t e0, e1;
  FSHT_CUDA_TRY(cudaEventCreate(&e0));
  FSHT_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    FSHT_CUDA_TRY(cudaEventRecord(e0, 0));
    k_umma_loop<N><<<nsm, 128, kUmmaProbeSmem>>>(iters, d_err);
    FSHT_LAUNCH_CHECK();
    FSHT_CUDA_TRY(cudaEventRecord(e1, 0));
    FSHT_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    FSHT_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *tflops = 2.0 * 128 * N * 16 * 10.0 * iters * nsm / (best * 1e-3) / 1e12;
  return FSHT_OK;
}
}  // namespace

extern "C" int fsht_measure_umma_rate(int n_cols, double* tflops) {
  if (!tflops || (n_cols != 128 && n_cols != 256)) {
    fsht_set_error("measure_umma_rate: n_cols must be 128 or 256");
    return FSHT_EINVAL;
  }
  int dev = 0, nsm = 0;
  FSHT_CUDA_TRY(cudaGetDevice(&dev));
  FSHT_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int* d_err = nullptr;
  FSHT_CUDA_TRY(cudaMalloc(&d_err, sizeof(int)));
  FSHT_CUDA_TRY(cudaMemset(d_err, 0, sizeof(int)));
  const int rc = n_cols == 128 ? umma_rate<128>(nsm, d_err, tflops)
                               : umma_rate<256>(nsm, d_err, tflops);
  int err = 0;
  cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d_err);
  if (rc) return rc;
  if (err) {
    fsht_set_error("measure_umma_rate: a wait expired");
    return FSHT_ETIMEOUT;
  }
  return FSHT_OK;
}
