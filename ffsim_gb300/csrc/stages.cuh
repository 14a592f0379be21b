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

// Diagonal operator of the fused expectation, seen from a stage whose rows
// are the member strings:  z(row, col) = zrow[row] + zcol[col]
//   + sum_{i, l} X[i][l] g_i(row) g_l(col),   g = n (number rep.) or 1 - 2n (Z rep.).
struct StageExpect {
  const float* zrow;
  const float* zcol;
  const unsigned* row_str;
  const unsigned* col_str;
  double* partials;  // one FP64 partial sum per CTA
  float X[FFGB_MAXN][FFGB_MAXN];
  float Xsum[FFGB_MAXN];  // sum_i X[i][l]
  int zrep;
};

struct WinStageParams {
  const float2* in;
  float2* out;      // unused by the fused expectation
  long long ld;     // row stride (elements)
  long long ncols;  // columns processed
  int n_classes;
  int cls_k[9];     // electrons inside the window, per class (largest classes first)
  int cls_cta0[10]; // first CTA of each class
  int cls_off[9];   // offset of the class's group bases (LOW) / member offsets (HIGH) in tab
  int tiles;        // column tiles per group
  int low;          // 1: window [0, h), members are consecutive rows after a per-group base row
  int norb, lo;     // orbitals; first orbital of the window
  int tab[256];
  float gp[84], gl[84];  // window network coefficients (see win_coef)
  unsigned gt[84];
  unsigned salt;
  const float2* ph_in;   // optional per-row phases applied before the network
  const float2* ph_out;  // optional per-row phases applied after the network
  StageExpect ex;
};

// Per-thread part of the fused expectation: the window orbitals' weights and
// the constant part of z for this (group, column).
struct ZCtx {
  float w[8];
  float base, scale;
  const float* zrow;
};

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// colex-ordered member j of a window with k of b orbitals occupied
__host__ __device__ constexpr unsigned win_member(int b, int k, int j) {
  unsigned m = 0;
  int count = 0;
  for (unsigned w = 0; w < (1u << b); ++w) {
    int pc = 0;
    for (unsigned x = w; x; x &= x - 1) ++pc;
    if (pc != k) continue;
    if (count == j) m = w;
    ++count;
  }
  return m;
}

template <int B, int K, int MODE, bool LOW>
static __device__ __noinline__ void win_rows(const float2* __restrict__ si, float2* __restrict__ so,
                                             long long ld, const int* __restrict__ off,
                                             const float* __restrict__ gp, const float* __restrict__ gl,
                                             const unsigned* __restrict__ gt, unsigned rng,
                                             const float2* __restrict__ ph_in,
                                             const float2* __restrict__ ph_out) {
  constexpr int M = WinNet<B, K>::M;
  float2 v[M];
#pragma unroll
  for (int j = 0; j < M; ++j) v[j] = si[(long long)(LOW ? j : off[j]) * ld];
  if (ph_in) {
#pragma unroll
    for (int j = 0; j < M; ++j) v[j] = cmulf(v[j], ph_in[LOW ? j : off[j]]);
  }
  WinNet<B, K>::template apply<MODE>(v, gp, gl, gt, rng);
  if (ph_out) {
#pragma unroll
    for (int j = 0; j < M; ++j) v[j] = cmulf(v[j], ph_out[LOW ? j : off[j]]);
  }
#pragma unroll
  for (int j = 0; j < M; ++j) so[(long long)(LOW ? j : off[j]) * ld] = v[j];
}

// Last stage fused with the expectation: returns sum_j z_j |v_j|^2 (FP32
// Kahan inside, FP64 out); nothing is stored.
template <int B, int K, int MODE, bool LOW>
static __device__ __noinline__ double win_rows_expect(const float2* __restrict__ si, long long ld,
                                                      const int* __restrict__ off, const float* __restrict__ gp,
                                                      const float* __restrict__ gl,
                                                      const unsigned* __restrict__ gt, unsigned rng, ZCtx z) {
  constexpr int M = WinNet<B, K>::M;
  float2 v[M];
#pragma unroll
  for (int j = 0; j < M; ++j) v[j] = si[(long long)(LOW ? j : off[j]) * ld];
  WinNet<B, K>::template apply<MODE>(v, gp, gl, gt, rng);
  float acc = 0.f, cmp = 0.f;
#pragma unroll
  for (int j = 0; j < M; ++j) {
    const unsigned mem = win_member(B, K, j);
    float wsum = 0.f;
#pragma unroll
    for (int t = 0; t < B; ++t)
      if ((mem >> t) & 1u) wsum += z.w[t];
    const float zj = __ldg(z.zrow + (LOW ? j : off[j])) + z.base + z.scale * wsum;
    const float y = zj * (v[j].x * v[j].x + v[j].y * v[j].y) - cmp;
    const float t2 = acc + y;
    cmp = (t2 - acc) - y;
    acc = t2;
  }
  return (double)acc - (double)cmp;
}

template <int B, int MODE, int K = 0>
__device__ __forceinline__ void win_rows_k(int k, bool low, const float2* si, float2* so, long long ld,
                                           const int* off, const float* gp, const float* gl, const unsigned* gt,
                                           unsigned rng, const float2* ph_in, const float2* ph_out) {
  if constexpr (K <= B) {
    if (k == K) {
      if (low)
        win_rows<B, K, MODE, true>(si, so, ld, off, gp, gl, gt, rng, ph_in, ph_out);
      else
        win_rows<B, K, MODE, false>(si, so, ld, off, gp, gl, gt, rng, ph_in, ph_out);
    } else {
      win_rows_k<B, MODE, K + 1>(k, low, si, so, ld, off, gp, gl, gt, rng, ph_in, ph_out);
    }
  }
}

template <int B, int MODE, int K = 0>
__device__ __forceinline__ double win_expect_k(int k, bool low, const float2* si, long long ld, const int* off,
                                               const float* gp, const float* gl, const unsigned* gt, unsigned rng,
                                               const ZCtx& z) {
  if constexpr (K <= B) {
    if (k == K) {
      return low ? win_rows_expect<B, K, MODE, true>(si, ld, off, gp, gl, gt, rng, z)
                 : win_rows_expect<B, K, MODE, false>(si, ld, off, gp, gl, gt, rng, z);
    }
    return win_expect_k<B, MODE, K + 1>(k, low, si, ld, off, gp, gl, gt, rng, z);
  } else {
    return 0.0;
  }
}

// Sum over the CTA's 128 threads; the result is valid in thread 0.
__device__ __forceinline__ double block_sum_128(double a, double* sh) {
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = a;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < STAGE_THREADS / 32; ++w) s += sh[w];
  return s;
}

template <int B, int MODE, bool EXPECT>
__global__ void __launch_bounds__(STAGE_THREADS, 2) win_stage_kernel(const __grid_constant__ WinStageParams P) {
  const int cta = blockIdx.x;
  int ci = 0;
  while (ci + 1 < P.n_classes && cta >= P.cls_cta0[ci + 1]) ++ci;
  const int k = P.cls_k[ci];
  const int local = cta - P.cls_cta0[ci];
  const int g = local / P.tiles, tile = local - g * P.tiles;
  const long long col = (long long)tile * STAGE_THREADS + threadIdx.x;
  const bool active = col < P.ncols;
  if (!EXPECT && !active) return;
  const bool low = P.low != 0;
  long long row0;
  const int* off;
  if (low) {
    row0 = P.tab[P.cls_off[ci] + g];
    off = nullptr;
  } else {
    row0 = g;
    off = P.tab + P.cls_off[ci];
  }
  const unsigned rng = dither_seed((unsigned long long)col, P.salt);
  if constexpr (!EXPECT) {
    const float2* si = P.in + row0 * P.ld + col;
    float2* so = P.out + row0 * P.ld + col;
    win_rows_k<B, MODE>(k, low, si, so, P.ld, off, P.gp, P.gl, P.gt, rng, P.ph_in ? P.ph_in + row0 : nullptr,
                        P.ph_out ? P.ph_out + row0 : nullptr);
  } else {
    __shared__ double sh[STAGE_THREADS / 32];
    double part = 0.0;
    if (active) {
      const StageExpect& E = P.ex;
      const unsigned cstr = E.col_str[col];
      // the orbitals outside the window are the same for every member: read member 0
      const unsigned r0str = E.row_str[row0 + (low ? 0 : off[0])];
      const unsigned wmask = ((1u << B) - 1u) << P.lo;
      const unsigned outside = r0str & ~wmask;
      ZCtx z;
      float s_out = 0.f, w_all = 0.f;
#pragma unroll
      for (int t = 0; t < B; ++t) z.w[t] = 0.f;
      for (int l = 0; l < P.norb; ++l) {
        const float gcol = E.zrep ? (((cstr >> l) & 1u) ? -1.f : 1.f) : (float)((cstr >> l) & 1u);
#pragma unroll
        for (int t = 0; t < B; ++t) z.w[t] += E.X[P.lo + t][l] * gcol;
        for (unsigned o = outside; o; o &= o - 1) s_out += E.X[__ffs(o) - 1][l] * gcol;
        w_all += E.Xsum[l] * gcol;
      }
      const float zc = E.zcol[col];
      if (E.zrep) {
        z.base = zc + w_all - 2.f * s_out;
        z.scale = -2.f;
      } else {
        z.base = zc + s_out;
        z.scale = 1.f;
      }
      z.zrow = E.zrow + row0;
      part = win_expect_k<B, MODE>(k, low, P.in + row0 * P.ld + col, P.ld, off, P.gp, P.gl, P.gt, rng, z);
    }
    const double s = block_sum_128(part, sh);
    if (threadIdx.x == 0) P.ex.partials[blockIdx.x] = s;
  }
}

// Cross-half rotations (i, h + i) of up to four sites in one pass.  A group is
// the set of strings that agree everywhere except in which orbital of each
// "active" pair (exactly one of i, h + i occupied) is occupied: 2^M members
// for M active sites.  Table entry per group: a header with the active sites
// (3 bits each, ascending), then per member its row | (sign bits << 24); bit
// 24 + t is the parity of the occupied orbitals strictly between the two
// orbitals of active site t, read on the member whose lower orbital is
// occupied.  Pairs with both or neither orbital occupied are left alone: the
// 2x2 blocks of the plan have determinant 1.
struct CsStageParams {
  float2* x;
  long long ld, ncols;
  const int* tab;
  int n_classes;
  int cls_m[5];
  int cls_cta0[6];
  int cls_base[5];  // first int of the class's groups in tab
  int tiles;
  float gp[24], gl[24];  // per site (c, Re t, Im t), see win_coef
  unsigned gt[24];
  unsigned salt;
};

template <int M, int MODE>
static __device__ __noinline__ void cs_group(float2* __restrict__ xc, long long ld, const int* __restrict__ ent,
                                             const float* __restrict__ gp, const float* __restrict__ gl,
                                             const unsigned* __restrict__ gt, unsigned rng) {
  constexpr int NM = 1 << M;
  const int sites = ent[0];
  int e[NM];
  float2 v[NM];
#pragma unroll
  for (int j = 0; j < NM; ++j) {
    e[j] = ent[1 + j];
    v[j] = xc[(long long)(e[j] & 0xffffff) * ld];
  }
#pragma unroll
  for (int t = 0; t < M; ++t) {
    const int site = (sites >> (3 * t)) & 7;
    float c, sr, si, cl, srl, sil;
    win_coef<MODE>(gp, gl, gt, site, rng, c, sr, si, cl, srl, sil);
#pragma unroll
    for (int j = 0; j < NM; ++j) {
      if (j & (1 << t)) continue;
      const float sg = ((e[j] >> (24 + t)) & 1) ? -1.f : 1.f;
      rot_pair<MODE == 1>(v[j], v[j | (1 << t)], c, sg * sr, sg * si, cl, sg * srl, sg * sil);
    }
  }
#pragma unroll
  for (int j = 0; j < NM; ++j) xc[(long long)(e[j] & 0xffffff) * ld] = v[j];
}

template <int MODE>
__global__ void __launch_bounds__(STAGE_THREADS, 2) cs_stage_kernel(const __grid_constant__ CsStageParams P) {
  const int cta = blockIdx.x;
  int ci = 0;
  while (ci + 1 < P.n_classes && cta >= P.cls_cta0[ci + 1]) ++ci;
  const int m = P.cls_m[ci];
  const int local = cta - P.cls_cta0[ci];
  const int g = local / P.tiles, tile = local - g * P.tiles;
  const long long col = (long long)tile * STAGE_THREADS + threadIdx.x;
  if (col >= P.ncols) return;
  const int* ent = P.tab + P.cls_base[ci] + (long long)g * (1 + (1 << m));
  const unsigned rng = dither_seed((unsigned long long)col, P.salt);
  float2* xc = P.x + col;
  switch (m) {
    case 1: cs_group<1, MODE>(xc, P.ld, ent, P.gp, P.gl, P.gt, rng); break;
    case 2: cs_group<2, MODE>(xc, P.ld, ent, P.gp, P.gl, P.gt, rng); break;
    case 3: cs_group<3, MODE>(xc, P.ld, ent, P.gp, P.gl, P.gt, rng); break;
    case 4: cs_group<4, MODE>(xc, P.ld, ent, P.gp, P.gl, P.gt, rng); break;
    default: break;
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
