// Definition of launch_sector; included by the instantiation units only.
#pragma once

#include "common.h"

namespace ffgb {

template <typename T, int NW>
int launch_sector(const SectorParams<T>& P, int grid, int block, int smem, cudaStream_t st) {
  static bool attr_set = false;  // one instantiation per (T, NW)
  if (!attr_set) {
    FFGB_CUDA(cudaFuncSetAttribute(sector_kernel<T, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   227 * 1024));
    attr_set = true;
  }
  sector_kernel<T, NW><<<grid, block, smem, st>>>(P);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

}  // namespace ffgb
