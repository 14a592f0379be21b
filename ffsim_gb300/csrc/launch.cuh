// Definition of launch_sector; included by the instantiation units only.
#pragma once

#include <atomic>

#include "common.h"

namespace ffgb {

template <typename T, int NW>
int launch_sector(const SectorParams<T>& P, long long n_chunks, int block, int smem, cudaStream_t st,
                  int* grid_out) {
  // per device: the shared-memory opt-in and the SM count
  static std::atomic<int> sms[64];
  int dev = 0;
  FFGB_CUDA(cudaGetDevice(&dev));
  int dev_sms = (dev >= 0 && dev < 64) ? sms[dev].load() : 0;
  if (dev_sms == 0) {
    FFGB_CUDA(cudaFuncSetAttribute(sector_kernel<T, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   227 * 1024));
    FFGB_CUDA(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, dev));
    if (dev >= 0 && dev < 64) sms[dev].store(dev_sms);
  }
  int per_sm = 0;
  FFGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sector_kernel<T, NW>, block, smem));
  if (per_sm < 1) return fail(FFGB_ERR_UNSUPPORTED, "sector kernel does not fit on an SM");
  const long long cap = (long long)per_sm * dev_sms;
  const int grid = (int)(n_chunks < cap ? n_chunks : cap);
  sector_kernel<T, NW><<<grid, block, smem, st>>>(P);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  if (grid_out) *grid_out = grid;
  return FFGB_OK;
}

}  // namespace ffgb
