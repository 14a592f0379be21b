// Launch of one window-stage job.  launch_win_bk<B, K> is instantiated by
// stage_inst.cu, compiled once per (B, range of K) for parallel builds.
#pragma once

#include "common.h"
#include "stages.cuh"

namespace ffgb {

template <int B, int K, int KIND>
int launch_win_job_k(const WinJob& P, bool low, int epi, long long items, cudaStream_t st, int* grid_used) {
  if (low && epi != EPI_STORE) return fail(FFGB_ERR_ARG, "the expectation runs on the upper window");
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
int launch_win_bk(const WinJob& P, int kind, bool low, int epi, long long items, cudaStream_t st, int* grid_used) {
  if (kind == 0) return launch_win_job_k<B, K, 0>(P, low, epi, items, st, grid_used);
  if constexpr (2 * K == B) {
    if (kind == 1) return launch_win_job_k<B, K, 1>(P, low, epi, items, st, grid_used);
  }
  if constexpr (2 * K < B && win_members(B, K) <= 35) {
    if (kind == 2) return launch_win_job_k<B, K, 2>(P, low, epi, items, st, grid_used);
  }
  return fail(FFGB_ERR_ARG, "no packed kernel for this window class");
}

}  // namespace ffgb
