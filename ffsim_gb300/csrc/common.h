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

// Message of the calling thread's last error (cleared at the start of every
// entry point).
extern thread_local std::string g_err;

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
  long long col_period = 0;  // stacked states: column c is string c mod col_period (0: one state)
  long long col_valid = 0;   // strings per state (columns col_valid..col_period-1 are zero padding)
};

struct StageOpts {
  int mode = 2;             // window coefficients: 0 plain FP32, 1 compensated, 2 dithered
  unsigned salt = 0;        // decorrelates the dithering of different rotations
  const StageExpectArgs* expect = nullptr;  // last stage reduces instead of storing
  int* expect_ctas = nullptr;               // partials written by the fused expectation
  int only_stage = -1;  // >= 0: run only this stage (0 B1, 1 B2, 2 cross-half, 3 A1, 4 A2), in place
  long long col_period = 0;  // stacked states: dither column c as column c mod col_period
};

// Stage-major complex64 rotation of the sector whose strings index the rows
// of a row-major array (ld elements per row, ncols columns processed):
// in -> out (in == out allowed).
int stage_rotate_rows(const void* in, void* out, int norb, int nocc, long long ld, long long ncols,
                      const SectorPlan& plan, const StageOpts& o, cudaStream_t st);

// Upper bound of the partial sums written by a fused expectation on a state
// of `rows` rows (the rotated sector's strings) and ncols columns.
long long stage_expect_partials(long long rows, long long ncols);

// States stacked side by side along the columns are padded to whole column
// tiles of the stage kernels, so that no tile holds two states.
constexpr long long STACK_TILE = 128;
inline long long stack_pad(long long n) { return (n + STACK_TILE - 1) / STACK_TILE * STACK_TILE; }

// Densities between two states (grad.cu); results summed on the host in FP64.
template <typename T>
int rdm1_rows(const void* x, const void* y, const unsigned* strings, int rows, int cols, int norb,
              void* partial_buf, size_t partial_bytes, std::vector<double>& out, cudaStream_t st, int nocc,
              const unsigned* sub, int n_sub);
template <typename T>
int pair_rows(const void* x, const void* y, const unsigned* rstr, const unsigned* cstr, int rows, int cols,
              int norb, void* partial_buf, size_t partial_bytes, std::vector<double>& rr, std::vector<double>& rc,
              cudaStream_t st);
// The same into device memory, without synchronizing: g_dev gets norb * norb
// complex values, sums_dev 2 * norb * norb (row-row, then row-column).
template <typename T>
int rdm1_rows_dev(const void* x, const void* y, const unsigned* strings, int rows, int cols, int norb,
                  void* partial_buf, size_t partial_bytes, double2* g_dev, cudaStream_t st, int nocc,
                  const unsigned* sub, int n_sub);
template <typename T>
int pair_rows_dev(const void* x, const void* y, const unsigned* rstr, const unsigned* cstr, int rows, int cols,
                  int norb, void* partial_buf, size_t partial_bytes, double2* sums_dev, cudaStream_t st);
size_t density_partial_bytes(int norb, long long rows);
size_t density_sub_bytes(int norb, long long n_sub, int nv);
template <typename T>
int launch_transpose(const void* in, void* out, long long rows, long long cols, const void* row_ph,
                     const void* col_ph, cudaStream_t st);
// The same for n_states states side by side along the columns: state b is
// columns [b * in_pad, b * in_pad + cols) of `in` (row stride n_states *
// in_pad) and becomes columns [b * out_pad, b * out_pad + rows) of `out`
// (row stride n_states * out_pad).  Padding columns are not written.
template <typename T>
int launch_transpose_stacked(const void* in, void* out, long long rows, long long cols, long long n_states,
                             long long in_pad, long long out_pad, const void* row_ph, cudaStream_t st);
// Contiguous states x[b] (rows x cols) <-> stacked y (pad columns per state):
// dir 0 x -> y, dir 1 y -> x (accumulate: x += y).
template <typename T>
int launch_stack(void* x, void* y, long long n_states, long long rows, long long cols, long long pad, int dir,
                 int accumulate, cudaStream_t st);
// Per-state sums of n per-CTA partials of a stacked stage (tiles column tiles
// per stage, tiles_per_state per state) into out[0..n_states).
int launch_state_partials(const double* partials, long long n, long long tiles, long long tiles_per_state,
                          long long n_states, double* out, cudaStream_t st);
template <typename T>
int launch_string_phases(const unsigned* strings, long long dim, int norb, const double* d_host, void* out,
                         cudaStream_t st);
template <typename T>
int launch_row_scale(void* x, long long rows, long long ld, const void* ph, cudaStream_t st);
template <typename T>
int launch_axpy(const void* x, void* y, long long n, double a, cudaStream_t st);
// y += ph[r] * x for rows r of length ld (ph nullptr: y += x).
template <typename T>
int launch_row_axpy(const void* x, void* y, long long rows, long long ld, const void* ph, cudaStream_t st);

}  // namespace ffgb
