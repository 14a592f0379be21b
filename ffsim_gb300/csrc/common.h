// Declarations shared by the translation units of libffgb.
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/ffsim_gb300.h"
#include "kernels.cuh"

namespace ffgb {

// Record an error message for ffgb_last_error() and return `code`.
int fail(int code, const std::string& msg);

// Count one kernel launch (reported by ffgb_launch_count()).
void count_launch();

#define FFGB_CUDA(call)                                                              \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return ::ffgb::fail(FFGB_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

#define FFGB_TRY(call)            \
  do {                            \
    int s_ = (call);              \
    if (s_ != FFGB_OK) return s_; \
  } while (0)

// Launch sector_kernel<T, NW>; instantiated in the inst_*.cu units.
template <typename T, int NW>
int launch_sector(const SectorParams<T>& P, int grid, int block, int smem, cudaStream_t st);

}  // namespace ffgb
