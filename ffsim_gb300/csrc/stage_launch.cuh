// Launch of one window stage; instantiated per window size in stage_b*.cu.
#pragma once

#include "common.h"
#include "stages.cuh"

namespace ffgb {

template <int B>
int launch_win_stage(const WinStageParams& P, int grid, int mode, bool expect, cudaStream_t st) {
  if (expect) {
    if (mode == 1)
      win_stage_kernel<B, 1, true><<<grid, STAGE_THREADS, 0, st>>>(P);
    else if (mode == 2)
      win_stage_kernel<B, 2, true><<<grid, STAGE_THREADS, 0, st>>>(P);
    else
      return fail(FFGB_ERR_ARG, "fused expectation needs compensated or dithered coefficients");
  } else {
    if (mode == 0)
      win_stage_kernel<B, 0, false><<<grid, STAGE_THREADS, 0, st>>>(P);
    else if (mode == 1)
      win_stage_kernel<B, 1, false><<<grid, STAGE_THREADS, 0, st>>>(P);
    else
      win_stage_kernel<B, 2, false><<<grid, STAGE_THREADS, 0, st>>>(P);
  }
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

}  // namespace ffgb
