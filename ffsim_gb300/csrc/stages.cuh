// Stage-major kernels for complex64 sectors with 9 <= norb <= 16.
//
// The state is viewed as a row-major array whose rows are the strings of
// the sector being rotated (the other sector runs along the contiguous
// columns).  Each kernel applies one stage of the cosine-sine plan to every
// column: a thread owns one (group, column) pair, so the lanes of a warp
// read 32 consecutive columns of the same member row (coalesced 256-byte
// accesses), every CTA runs a single electron-count class (one code path
// per CTA, no barriers), and a stage is one read and one write of the
// state.
#pragma once

#include "kernels.cuh"

namespace ffgb {

constexpr int STAGE_THREADS = 128;

struct WinStageParams {
  const float2* in;
  float2* out;
  long long ld;     // row stride (elements)
  long long ncols;  // columns processed
  int n_classes;
  int cls_k[9];     // electrons inside the window, per class (largest classes first)
  int cls_cta0[10]; // first CTA of each class
  int cls_off[9];   // offset of the class's group bases (LOW) / member offsets (HIGH) in tab
  int tiles;        // column tiles per group
  int low;          // 1: members are consecutive rows after a per-group base row
  int tab[256];
  int ident[72];
  float gp[84], gl[84];  // window network coefficients (c, Re s, Im s) and FP32 residuals
  int comp;
  const float2* ph_in;   // optional per-row phases applied before the network
  const float2* ph_out;  // optional per-row phases applied after the network
};

template <int B>
__global__ void __launch_bounds__(STAGE_THREADS, 2)
    win_stage_kernel(const __grid_constant__ WinStageParams P) {
  const int cta = blockIdx.x;
  int ci = 0;
  while (ci + 1 < P.n_classes && cta >= P.cls_cta0[ci + 1]) ++ci;
  const int k = P.cls_k[ci];
  const int local = cta - P.cls_cta0[ci];
  const int g = local / P.tiles, tile = local - g * P.tiles;
  const long long col = (long long)tile * STAGE_THREADS + threadIdx.x;
  if (col >= P.ncols) return;
  long long row0;
  const int* off;
  if (P.low) {
    row0 = P.tab[P.cls_off[ci] + g];
    off = P.ident;
  } else {
    row0 = g;
    off = P.tab + P.cls_off[ci];
  }
  const float2* si = P.in + row0 * P.ld + col;
  float2* so = P.out + row0 * P.ld + col;
  const float2* pin = P.ph_in ? P.ph_in + row0 : nullptr;
  const float2* pout = P.ph_out ? P.ph_out + row0 : nullptr;
  if (P.comp)
    WinDispatch<B>::template rows<true>(k, si, so, P.ld, off, P.gp, P.gl, pin, pout);
  else
    WinDispatch<B>::template rows<false>(k, si, so, P.ld, off, P.gp, P.gl, pin, pout);
}

struct CsSiteParams {
  float2* x;
  long long ld, ncols;
  const int* pairs;  // per pair: x_row | (fermionic sign bit << 31), y_row
  int n_pairs, ppc, tiles;
  float g[8], gl[8];  // [[g00, g01], [g10, g11]] (re, im) and FP32 residuals
  int comp;
};

// One cross-half rotation (i, H + i): x <- g00 x + sgn g01 y, y <- sgn g10 x + g11 y.
__global__ void __launch_bounds__(STAGE_THREADS) cs_site_kernel(const __grid_constant__ CsSiteParams P) {
  const int tile = blockIdx.x % P.tiles, chunk = blockIdx.x / P.tiles;
  const long long col = (long long)tile * STAGE_THREADS + threadIdx.x;
  if (col >= P.ncols) return;
  const int p0 = chunk * P.ppc;
  const int p1 = min(p0 + P.ppc, P.n_pairs);
  const bool comp = P.comp != 0;
  for (int p = p0; p < p1; ++p) {
    const int xe = P.pairs[2 * p], yr = P.pairs[2 * p + 1];
    const float sgn = xe < 0 ? -1.f : 1.f;
    const long long xr = xe & 0x7fffffff;
    float2* px = P.x + xr * P.ld + col;
    float2* py = P.x + (long long)yr * P.ld + col;
    const float2 x = *px, y = *py;
    float ax = 0.f, ay = 0.f, bx = 0.f, by = 0.f;
    if (comp) {
      ax = P.gl[0] * x.x - P.gl[1] * x.y + sgn * (P.gl[2] * y.x - P.gl[3] * y.y);
      ay = P.gl[0] * x.y + P.gl[1] * x.x + sgn * (P.gl[2] * y.y + P.gl[3] * y.x);
      bx = sgn * (P.gl[4] * x.x - P.gl[5] * x.y) + P.gl[6] * y.x - P.gl[7] * y.y;
      by = sgn * (P.gl[4] * x.y + P.gl[5] * x.x) + P.gl[6] * y.y + P.gl[7] * y.x;
    }
    float2 nx, ny;
    nx.x = P.g[0] * x.x - P.g[1] * x.y + sgn * (P.g[2] * y.x - P.g[3] * y.y) + ax;
    nx.y = P.g[0] * x.y + P.g[1] * x.x + sgn * (P.g[2] * y.y + P.g[3] * y.x) + ay;
    ny.x = sgn * (P.g[4] * x.x - P.g[5] * x.y) + P.g[6] * y.x - P.g[7] * y.y + bx;
    ny.y = sgn * (P.g[4] * x.y + P.g[5] * x.x) + P.g[6] * y.y + P.g[7] * y.x + by;
    *px = nx;
    *py = ny;
  }
}

// out[c][r] = in[r][c] * row_ph[r] * col_ph[c] (phase tables optional).
template <typename C>
__global__ void __launch_bounds__(256) transpose_kernel(const C* __restrict__ in, C* __restrict__ out,
                                                        long long rows, long long cols,
                                                        const C* __restrict__ row_ph,
                                                        const C* __restrict__ col_ph) {
  __shared__ C tile[32][33];
  const long long c0 = (long long)blockIdx.x * 32, r0 = (long long)blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int j = ty; j < 32; j += 8) {
    const long long r = r0 + j, c = c0 + tx;
    if (r < rows && c < cols) {
      C v = in[r * cols + c];
      if (row_ph) v = cmul(v, row_ph[r]);
      if (col_ph) v = cmul(v, col_ph[c]);
      tile[j][tx] = v;
    }
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const long long c = c0 + j, r = r0 + tx;
    if (c < cols && r < rows) out[c * rows + r] = tile[tx][j];
  }
}

struct OrbPhases {
  double d[2 * FFGB_MAXN];  // (re, im) per orbital
};

// Per-string phase prod_{i in occ(s)} d_i (final orbital phases of a plan).
template <typename C>
__global__ void string_phase_kernel(const unsigned* __restrict__ strings, long long dim, int norb,
                                    const __grid_constant__ OrbPhases D, C* __restrict__ out) {
  const double* d = D.d;
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j >= dim) return;
  const unsigned s = strings[j];
  double re = 1.0, im = 0.0;
  for (int i = 0; i < norb; ++i)
    if ((s >> i) & 1u) {
      const double a = re * d[2 * i] - im * d[2 * i + 1];
      const double b = re * d[2 * i + 1] + im * d[2 * i];
      re = a;
      im = b;
    }
  out[j] = cmake<C>(re, im);
}

// rows of x (row length ld) scaled by per-row phases
template <typename C>
__global__ void row_scale_kernel(C* __restrict__ x, long long rows, long long ld, const C* __restrict__ ph) {
  const long long n = rows * ld;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] = cmul(x[i], ph[i / ld]);
}

// y += a * x
template <typename T>
__global__ void axpy_kernel(const typename CT<T>::type* __restrict__ x, typename CT<T>::type* __restrict__ y,
                            long long n, T ar, T ai) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const typename CT<T>::type v = x[i];
    typename CT<T>::type o = y[i];
    o.x += ar * v.x - ai * v.y;
    o.y += ar * v.y + ai * v.x;
    y[i] = o;
  }
}

}  // namespace ffgb
