// Launch of one window-stage job.  launch_win_bk<B, K> is instantiated by
// stage_inst.cu, compiled once per (B, range of K) for parallel builds.
#pragma once

#include <algorithm>

#include "common.h"
#include "stages.cuh"

namespace ffgb {

inline int stage_num_sms() {
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 132;
  }();
  return sms;
}

// Pipelined kernel: a persistent grid of as many CTAs as fit on the device.
template <int B, int K, int KIND, bool LOW, int EPI>
int launch_tma(const WinJob& P, long long items, cudaStream_t st, int* grid_used) {
  constexpr int smem = win_slots<B, K, KIND>() * STAGE_THREADS * (int)sizeof(float2);
  static const int bps = [] {
    cudaFuncSetAttribute(win_tma_kernel<B, K, KIND, LOW, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    // the whole unified L1 as shared memory: two CTAs of ~72 KB per SM
    cudaFuncSetAttribute(win_tma_kernel<B, K, KIND, LOW, EPI>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, win_tma_kernel<B, K, KIND, LOW, EPI>, STAGE_THREADS, smem);
    return std::max(b, 1);
  }();
  const long long grid = std::min<long long>(items, (long long)stage_num_sms() * bps);
  if (grid <= 0) {
    *grid_used = 0;
    return FFGB_OK;
  }
  win_tma_kernel<B, K, KIND, LOW, EPI><<<(unsigned)grid, STAGE_THREADS, smem, st>>>(P);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  *grid_used = (int)grid;
  return FFGB_OK;
}

template <int B, int K, int KIND>
int launch_win_job_k(const WinJob& P, bool low, int epi, bool tma, long long items, cudaStream_t st,
                     int* grid_used) {
  if (low && epi != EPI_STORE) return fail(FFGB_ERR_ARG, "the expectation runs on the upper window");
  if (tma) {
    if (low) return launch_tma<B, K, KIND, true, EPI_STORE>(P, items, st, grid_used);
    if (epi == EPI_STORE) return launch_tma<B, K, KIND, false, EPI_STORE>(P, items, st, grid_used);
    return launch_tma<B, K, KIND, false, EPI_EXPECT>(P, items, st, grid_used);
  }
  const unsigned grid = (unsigned)items;
  if (low) {
    win_class_kernel<B, K, KIND, true, EPI_STORE><<<grid, STAGE_THREADS, 0, st>>>(P);
  } else if (epi == EPI_STORE) {
    win_class_kernel<B, K, KIND, false, EPI_STORE><<<grid, STAGE_THREADS, 0, st>>>(P);
  } else {
    win_class_kernel<B, K, KIND, false, EPI_EXPECT><<<grid, STAGE_THREADS, 0, st>>>(P);
  }
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  *grid_used = (int)grid;
  return FFGB_OK;
}

// kind 0: plain members; 1: K = B/2 complement-packed; 2: classes K and B - K packed together
template <int B, int K>
int launch_win_bk(const WinJob& P, int kind, bool low, int epi, bool tma, long long items, cudaStream_t st,
                  int* grid_used) {
  if (kind == 0) return launch_win_job_k<B, K, 0>(P, low, epi, tma, items, st, grid_used);
  if constexpr (2 * K == B) {
    if (kind == 1) return launch_win_job_k<B, K, 1>(P, low, epi, tma, items, st, grid_used);
  }
  if constexpr (2 * K < B && win_members(B, K) <= 35) {
    if (kind == 2) return launch_win_job_k<B, K, 2>(P, low, epi, tma, items, st, grid_used);
  }
  return fail(FFGB_ERR_ARG, "no packed kernel for this window class");
}

}  // namespace ffgb
