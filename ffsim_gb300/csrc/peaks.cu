// Arithmetic ceilings measured in-process: the FP64 and FP32 fused
// multiply-add rate of the CUDA cores, the denominators of the complex128 and
// complex64 rotation kernels' compute rooflines.  Each thread runs eight
// independent FMA chains (enough to cover the pipeline latency), the grid is
// a whole number of waves over the SMs, and the time is taken with CUDA
// events on the caller's stream.
#include <cuda_runtime.h>

#include "common.h"

namespace ffgb {

constexpr int PEAK_CHAINS = 8;
constexpr int PEAK_THREADS = 256;

// Where a chain's result would go: a data-dependent store keeps the compiler
// from removing the chains, and no input used here ever takes it.
__device__ double g_fma_sink;

template <typename T>
__global__ void __launch_bounds__(PEAK_THREADS) fma_chain_kernel(int iters, T a, T b) {
  T x[PEAK_CHAINS];
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = (T)(threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
#pragma unroll
      for (int c = 0; c < PEAK_CHAINS; ++c) x[c] = x[c] * a + b;
    }
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; ++c) s += x[c];
  if (s == (T)-1.2345e-30) g_fma_sink = (double)s;
}

}  // namespace ffgb

using namespace ffgb;

extern "C" int ffgb_debug_fma_rate(int dtype, double* tflops, void* stream) {
  if (!tflops) return fail(FFGB_ERR_ARG, "tflops is NULL");
  if (dtype != FFGB_C64 && dtype != FFGB_C128) return fail(FFGB_ERR_DTYPE, "dtype must be FFGB_C64 or FFGB_C128");
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0, per_sm = 0;
  FFGB_CUDA(cudaGetDevice(&dev));
  FFGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const bool f64 = dtype == FFGB_C128;
  if (f64)
    FFGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_chain_kernel<double>, PEAK_THREADS, 0));
  else
    FFGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_chain_kernel<float>, PEAK_THREADS, 0));
  const int grid = sms * (per_sm > 0 ? per_sm : 1) * 4;
  // FP64 on this part is slow: fewer iterations keep the launch near 10 ms
  const int iters = f64 ? 64 : 2048;
  cudaEvent_t a = nullptr, b = nullptr;
  FFGB_CUDA(cudaEventCreate(&a));
  FFGB_CUDA(cudaEventCreate(&b));
  float ms = 0.f;
  for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
    FFGB_CUDA(cudaEventRecord(a, st));
    if (f64)
      fma_chain_kernel<double><<<grid, PEAK_THREADS, 0, st>>>(iters, 0.999999, 1e-7);
    else
      fma_chain_kernel<float><<<grid, PEAK_THREADS, 0, st>>>(iters, 0.9999f, 1e-4f);
    count_launch();
    FFGB_CUDA(cudaGetLastError());
    FFGB_CUDA(cudaEventRecord(b, st));
    FFGB_CUDA(cudaEventSynchronize(b));
    FFGB_CUDA(cudaEventElapsedTime(&ms, a, b));
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  const double flops = 2.0 * (double)grid * PEAK_THREADS * PEAK_CHAINS * 16.0 * (double)iters;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return FFGB_OK;
}
