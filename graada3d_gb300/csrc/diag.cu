// FP64 fused-multiply-add throughput of the device: the denominator for the
// assembly kernel's roofline (the prism kernel is bound by the FP64 pipe).
// Eight independent DFMA chains per thread keep the pipe busy without memory
// traffic; the chains are contracting (|a| < 1) so values stay finite.
#include "common.cuh"
#include "kernels.h"

namespace grada {

namespace {

constexpr int PK_THREADS = 256;
constexpr int PK_CHAINS = 8;

__global__ void __launch_bounds__(PK_THREADS) dfma_loop_kernel(double *out, int iters, double a,
                                                               double b) {
  double x[PK_CHAINS];
#pragma unroll
  for (int c = 0; c < PK_CHAINS; c++) x[c] = (threadIdx.x + c) * 1e-3;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < PK_CHAINS; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < PK_CHAINS; c++) s += x[c];
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the loop alive, never true
}

}  // namespace

double measure_fp64_fma_rate(int sm_count, cudaStream_t s) {
  double *d_out = nullptr;
  GRADA_CUDA_CHECK(cudaMallocAsync(&d_out, sizeof(double) * 4096, s));
  const int blocks = sm_count * 8;
  const int iters = 2048;
  cudaEvent_t e0, e1;
  GRADA_CUDA_CHECK(cudaEventCreate(&e0));
  GRADA_CUDA_CHECK(cudaEventCreate(&e1));
  dfma_loop_kernel<<<blocks, PK_THREADS, 0, s>>>(d_out, iters, 0.999999, 1e-7);  // warm-up
  GRADA_LAUNCH_CHECK();
  float best_ms = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    GRADA_CUDA_CHECK(cudaEventRecord(e0, s));
    dfma_loop_kernel<<<blocks, PK_THREADS, 0, s>>>(d_out, iters, 0.999999, 1e-7);
    GRADA_LAUNCH_CHECK();
    GRADA_CUDA_CHECK(cudaEventRecord(e1, s));
    GRADA_CUDA_CHECK(cudaEventSynchronize(e1));
    float ms = 0.f;
    GRADA_CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) best_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  GRADA_CUDA_CHECK(cudaFreeAsync(d_out, s));
  GRADA_CUDA_CHECK(cudaStreamSynchronize(s));
  const double fmas = (double)blocks * PK_THREADS * iters * PK_CHAINS;
  return 2.0 * fmas / (best_ms * 1e-3);
}

}  // namespace grada
