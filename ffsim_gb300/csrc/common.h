// Declarations shared by the translation units of libffgb.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/ffsim_gb300.h"
#include "kernels.cuh"

namespace ffgb {

// Record an error message for ffgb_last_error() and return `code`.
int fail(int code, const std::string& msg);

// Count one kernel launch (reported by ffgb_launch_count()).
void count_launch();

// Count one device allocation made by the library (reported by
// ffgb_device_alloc_count()).
void count_alloc();

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

// Launch sector_kernel<T, NW> with a persistent grid of at most n_chunks CTAs
// (as many as fit on the device); the grid used is returned in *grid_out.
// Instantiated in the inst_*.cu units.
template <typename T, int NW>
int launch_sector(const SectorParams<T>& P, long long n_chunks, int block, int smem, cudaStream_t st,
                  int* grid_out);

struct SectorPlan;

// Fused expectation on the last stage of a stage-major rotation (see
// StageExpect in stages.cuh): sum z(row, col) |psi|^2 into one FP64 partial
// per CTA.  X[i][l] couples row orbital i with column orbital l.
struct StageExpectArgs {
  const float* zrow = nullptr;
  const float* zcol = nullptr;
  const unsigned* row_str = nullptr;
  const unsigned* col_str = nullptr;
  double* partials = nullptr;
  long long partial_cap = 0;
  float X[FFGB_MAXN][FFGB_MAXN] = {};
  int zrep = 0;
};

struct StageOpts {
  int mode = 2;             // window coefficients: 0 plain FP32, 1 compensated, 2 dithered
  unsigned salt = 0;        // decorrelates the dithering of different rotations
  const StageExpectArgs* expect = nullptr;  // last stage reduces instead of storing
  int* expect_ctas = nullptr;               // partials written by the fused expectation
  int only_stage = -1;  // >= 0: run only this stage (0 B1, 1 B2, 2 cross-half, 3 A1, 4 A2), in place
};

// Stage-major complex64 rotation of the sector whose strings index the rows
// of a row-major array (ld elements per row, ncols columns processed):
// in -> out (in == out allowed).
int stage_rotate_rows(const void* in, void* out, int norb, int nocc, long long ld, long long ncols,
                      const SectorPlan& plan, const StageOpts& o, cudaStream_t st);

// Upper bound of the partial sums written by a fused expectation on a state
// of `rows` rows (the rotated sector's strings) and ncols columns.
long long stage_expect_partials(long long rows, long long ncols);

// Densities between two states (grad.cu); results summed on the host in FP64.
template <typename T>
int rdm1_rows(const void* x, const void* y, const unsigned* strings, int rows, int cols, int norb,
              void* partial_buf, size_t partial_bytes, std::vector<double>& out, cudaStream_t st);
template <typename T>
int pair_rows(const void* x, const void* y, const unsigned* rstr, const unsigned* cstr, int rows, int cols,
              int norb, void* partial_buf, size_t partial_bytes, std::vector<double>& rr, std::vector<double>& rc,
              cudaStream_t st);
size_t density_partial_bytes(int norb, long long rows);
template <typename T>
int launch_transpose(const void* in, void* out, long long rows, long long cols, const void* row_ph,
                     const void* col_ph, cudaStream_t st);
template <typename T>
int launch_string_phases(const unsigned* strings, long long dim, int norb, const double* d_host, void* out,
                         cudaStream_t st);
template <typename T>
int launch_row_scale(void* x, long long rows, long long ld, const void* ph, cudaStream_t st);
template <typename T>
int launch_axpy(const void* x, void* y, long long n, double a, cudaStream_t st);

}  // namespace ffgb
