// Reduced densities between two states, for the adjoint gradient of the LUCJ
// energy:
//   transition one-body density  G^s_pq = <x| a+_{p s} a_{q s} |y>
//   diagonal pair density        P^{st}_ij = <x| n_{i s} n_{j t} |y>
// A thread sums its share of one row (a few dozen products) in the state's
// precision -- FP32 for complex64, whose products are FP32 anyway, FP64 for
// complex128 -- and everything above that (rows, CTAs) accumulates in FP64;
// the CTAs' partial sums are reduced on the host in a fixed order.  (FP64
// arithmetic per element ran at 3 GB/s on GB300, whose FP64 rate is low.)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.h"

namespace ffgb {

namespace {

constexpr int DTHREADS = 256;
constexpr int RDM_ROWS = 16;  // rows of the rotated sector per CTA

// Row partials in the state's precision: float2 for complex64, double2 for complex128.
template <typename C>
__device__ __forceinline__ C cdot_row(C acc, C a, C b) {  // acc += conj(a) * b
  acc.x = fma(a.x, b.x, fma(a.y, b.y, acc.x));
  acc.y = fma(a.x, b.y, fma(-a.y, b.x, acc.y));
  return acc;
}

template <typename C>
__device__ __forceinline__ double2 to_d2(C v) {
  return make_double2((double)v.x, (double)v.y);
}

__device__ __forceinline__ double2 block_sum2(double2 v, double2* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double2 s = make_double2(0.0, 0.0);
  if (threadIdx.x == 0)
    for (int w = 0; w < DTHREADS / 32; ++w) {
      s.x += sh[w].x;
      s.y += sh[w].y;
    }
  __syncthreads();
  return s;
}

// One (p, q) pair (blockIdx.y) over a chunk of rows (blockIdx.x) of the rotated
// sector, whose strings index the rows; columns = the other sector.
template <typename T>
__global__ void __launch_bounds__(DTHREADS) rdm1_kernel(const typename CT<T>::type* __restrict__ x,
                                                        const typename CT<T>::type* __restrict__ y,
                                                        const unsigned* __restrict__ strings, int rows, int cols,
                                                        int norb, double2* __restrict__ partial) {
  __shared__ int sB[FFGB_BST * FFGB_BST];
  __shared__ double2 sh[DTHREADS / 32];
  for (int idx = threadIdx.x; idx < FFGB_BST * FFGB_BST; idx += DTHREADS) {
    const int a = idx / FFGB_BST, b = idx % FFGB_BST;
    long long r = 0;
    if (b <= a) {
      r = 1;
      for (int i = 1; i <= b; ++i) r = r * (a - b + i) / i;
    }
    sB[idx] = (int)r;
  }
  __syncthreads();
  const int pair = blockIdx.y, p = pair / norb, q = pair - p * norb;
  const int a0 = blockIdx.x * RDM_ROWS, a1 = min(a0 + RDM_ROWS, rows);
  double2 acc = make_double2(0.0, 0.0);
  for (int a = a0; a < a1; ++a) {
    const unsigned s = strings[a];
    if (!((s >> q) & 1u)) continue;
    unsigned t = s;
    int sign = 0;
    if (p != q) {
      if ((s >> p) & 1u) continue;
      const unsigned r1 = s & ~(1u << q);
      sign = (__popc(s & ((1u << q) - 1u)) + __popc(r1 & ((1u << p) - 1u))) & 1;
      t = r1 | (1u << p);
    }
    const long long ap = rank_colex(t, sB);
    const auto* xr = x + ap * cols;
    const auto* yr = y + (long long)a * cols;
    typename CT<T>::type dr;
    dr.x = dr.y = (T)0;
    for (int c = threadIdx.x; c < cols; c += DTHREADS) dr = cdot_row(dr, xr[c], yr[c]);
    double2 d = to_d2(dr);
    if (sign) {
      d.x = -d.x;
      d.y = -d.y;
    }
    acc.x += d.x;
    acc.y += d.y;
  }
  const double2 s = block_sum2(acc, sh);
  if (threadIdx.x == 0) partial[(long long)pair * gridDim.x + blockIdx.x] = s;
}

// The same density from the strings with one electron fewer: for every
// (n-1)-string s and column c,
//   G_pq += conj(sg_p(s) x[s + p][c]) sg_q(s) y[s + q][c]   (p, q not in s),
// sg_p(s) = (-1)^(electrons of s below p) the sign of a_p on s + p.  One CTA
// per s holds the (NV x NV) block over the vacancies of s (NV = norb - n + 1),
// so every row is read n times instead of once per (p, q) pair; the CTA's
// block goes to partial[s] (FP64) and rdm1_sub_reduce_kernel sums the blocks
// into G in a fixed order.  complex64 states, per-thread sums in FP32.
// NI = rows of the block per CTA: the block's rows [blockIdx.y * NI, ...) (all
// NV rows in one CTA when NI == NV; two CTAs for large NV, which would spill).
template <int NV, int NI>
__global__ void __launch_bounds__(DTHREADS) rdm1_sub_kernel(const float2* __restrict__ x,
                                                            const float2* __restrict__ y,
                                                            const unsigned* __restrict__ sub, int cols, int norb,
                                                            double2* __restrict__ partial) {
  __shared__ int sB[FFGB_BST * FFGB_BST];
  __shared__ long long srow[NV];
  __shared__ float ssg[NV];
  for (int idx = threadIdx.x; idx < FFGB_BST * FFGB_BST; idx += DTHREADS) {
    const int a = idx / FFGB_BST, b = idx % FFGB_BST;
    long long r = 0;
    if (b <= a) {
      r = 1;
      for (int i = 1; i <= b; ++i) r = r * (a - b + i) / i;
    }
    sB[idx] = (int)r;
  }
  __syncthreads();
  const unsigned s = sub[blockIdx.x];
  if (threadIdx.x < NV) {  // the j-th vacancy of s, its row and sign
    int v = -1;
    for (int o = 0, k = 0; o < norb; ++o)
      if (!((s >> o) & 1u)) {
        if (k == (int)threadIdx.x) {
          v = o;
          break;
        }
        ++k;
      }
    srow[threadIdx.x] = (long long)rank_colex(s | (1u << v), sB) * cols;
    ssg[threadIdx.x] = (__popc(s & ((1u << v) - 1u)) & 1) ? -1.f : 1.f;
  }
  __syncthreads();
  const int i0 = blockIdx.y * NI;
  float2 acc[NI][NV];
#pragma unroll
  for (int i = 0; i < NI; ++i)
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[i][j] = make_float2(0.f, 0.f);
  for (int c = threadIdx.x; c < cols; c += DTHREADS) {
    float2 xv[NI], yv[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const float2 b = y[srow[j] + c];
      yv[j] = make_float2(ssg[j] * b.x, ssg[j] * b.y);
    }
#pragma unroll
    for (int i = 0; i < NI; ++i) {
      if (i0 + i < NV) {  // uniform over the CTA
        const float2 a = x[srow[i0 + i] + c];
        xv[i] = make_float2(ssg[i0 + i] * a.x, ssg[i0 + i] * a.y);
      } else {
        xv[i] = make_float2(0.f, 0.f);
      }
    }
#pragma unroll
    for (int i = 0; i < NI; ++i)
#pragma unroll
      for (int j = 0; j < NV; ++j) acc[i][j] = cdot_row(acc[i][j], xv[i], yv[j]);
  }
  // every warp sums its lanes' blocks, then one thread per entry sums the
  // warps (fixed order): one barrier for the whole block
  __shared__ double2 wsum[DTHREADS / 32][NI * NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NI; ++i)
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double2 v = to_d2(acc[i][j]);
      for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
      }
      if (lane == 0) wsum[warp][i * NV + j] = v;
    }
  __syncthreads();
  double2* out = partial + (long long)blockIdx.x * NV * NV;
  for (int e = threadIdx.x; e < NI * NV; e += DTHREADS) {
    const int i = e / NV, j = e - i * NV;
    if (i0 + i >= NV) continue;
    double2 t = make_double2(0.0, 0.0);
    for (int w = 0; w < DTHREADS / 32; ++w) {
      t.x += wsum[w][e].x;
      t.y += wsum[w][e].y;
    }
    out[(i0 + i) * NV + j] = t;
  }
}

// Small sectors (the state a few MB, in L2): the same (NV x NV) block per
// (n-1)-string s as rdm1_sub_kernel, one CTA per s, one warp per entry of
// the block at a time (lanes over the columns, sums in FP32 per lane and
// FP64 across the warp by shuffles, no block barrier); rows are read from L2
// by the NV warps that need them.
__device__ __forceinline__ long long binom_ll(int n, int k) {
  if (k < 0 || k > n) return 0;
  long long r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

template <int NV>
__global__ void __launch_bounds__(DTHREADS) rdm1_small_kernel(const float2* __restrict__ x,
                                                              const float2* __restrict__ y,
                                                              const unsigned* __restrict__ sub, int cols, int norb,
                                                              double2* __restrict__ partial) {
  __shared__ long long srow[NV];
  __shared__ float ssg[NV];
  const unsigned s = sub[blockIdx.x];
  if (threadIdx.x < NV) {  // the j-th vacancy of s, its row and sign
    int v = -1;
    for (int o = 0, k = 0; o < norb; ++o)
      if (!((s >> o) & 1u)) {
        if (k == (int)threadIdx.x) {
          v = o;
          break;
        }
        ++k;
      }
    unsigned t = s | (1u << v);
    long long r = 0;
    for (int k = 1; t; ++k) {  // colex rank
      const int pos = __ffs(t) - 1;
      t &= t - 1;
      r += binom_ll(pos, k);
    }
    srow[threadIdx.x] = r * cols;
    ssg[threadIdx.x] = (__popc(s & ((1u << v) - 1u)) & 1) ? -1.f : 1.f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double2* out = partial + (long long)blockIdx.x * NV * NV;
  for (int e = warp; e < NV * NV; e += DTHREADS / 32) {
    const int i = e / NV, j = e - i * NV;
    const float2* xr = x + srow[i];
    const float2* yr = y + srow[j];
    float2 acc = make_float2(0.f, 0.f);
    for (int c = lane; c < cols; c += 32) acc = cdot_row(acc, xr[c], yr[c]);
    double2 v = to_d2(acc);
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, o);
      v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    if (lane == 0) {
      const double sg = (double)(ssg[i] * ssg[j]);
      out[e] = make_double2(sg * v.x, sg * v.y);
    }
  }
}

// G_pq = sum over the (n-1)-strings s with p, q not in s of block[s][i][j],
// i / j the positions of p / q among the vacancies of s; one CTA per (p, q),
// fixed order.
__global__ void __launch_bounds__(DTHREADS) rdm1_sub_reduce_kernel(const double2* __restrict__ partial,
                                                                   const unsigned* __restrict__ sub, int n_sub,
                                                                   int nv, int norb, double2* __restrict__ g) {
  __shared__ double2 sh[DTHREADS / 32];
  const int p = blockIdx.x / norb, q = blockIdx.x - p * norb;
  double2 a = make_double2(0.0, 0.0);
  for (int t = threadIdx.x; t < n_sub; t += DTHREADS) {
    const unsigned s = sub[t];
    if (((s >> p) & 1u) || ((s >> q) & 1u)) continue;
    const int i = p - __popc(s & ((1u << p) - 1u)), j = q - __popc(s & ((1u << q) - 1u));
    const double2 v = partial[(long long)t * nv * nv + i * nv + j];
    a.x += v.x;
    a.y += v.y;
  }
  const double2 r = block_sum2(a, sh);
  if (threadIdx.x == 0) g[blockIdx.x] = r;
}

template <int NV>
int launch_rdm1_sub(const void* x, const void* y, const unsigned* sub, int n_sub, int cols, int norb,
                    double2* partial, double2* g, bool small, cudaStream_t st) {
  constexpr int NI = NV >= 7 ? 3 : NV;  // at most 3 x 10 accumulators: two CTAs per SM
  if (small) {
    rdm1_small_kernel<NV><<<(unsigned)n_sub, DTHREADS, 0, st>>>((const float2*)x, (const float2*)y, sub, cols,
                                                                norb, partial);
  } else {
    const dim3 grid((unsigned)n_sub, (unsigned)((NV + NI - 1) / NI));
    rdm1_sub_kernel<NV, NI><<<grid, DTHREADS, 0, st>>>((const float2*)x, (const float2*)y, sub, cols, norb,
                                                       partial);
  }
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  rdm1_sub_reduce_kernel<<<norb * norb, DTHREADS, 0, st>>>(partial, sub, n_sub, NV, norb, g);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

// Pair densities within the row sector (P^rr_ij, rows i, j) and between the
// row and column sectors (P^rc_ij) over a chunk of PAIR_ROWS rows, one row per
// warp: per row the lanes sum w = conj(x) y over their columns (in the
// state's precision), in total and per occupied column orbital, reduce across
// the warp in FP64 by shuffles (no block barrier), and add the row's terms to
// the warp's own FP64 accumulators in shared memory; the CTA then sums its
// warps in a fixed order.
constexpr int PAIR_THREADS = 128;
constexpr int PAIR_ROWS = PAIR_THREADS / 32;

template <typename T>
__global__ void __launch_bounds__(PAIR_THREADS) pair_density_kernel(const typename CT<T>::type* __restrict__ x,
                                                                    const typename CT<T>::type* __restrict__ y,
                                                                    const unsigned* __restrict__ rstr,
                                                                    const unsigned* __restrict__ cstr, int rows,
                                                                    int cols, int norb,
                                                                    double2* __restrict__ partial) {
  using Cx = typename CT<T>::type;
  constexpr int NW = PAIR_THREADS / 32;
  __shared__ double2 acc_rr[NW][FFGB_MAXN * FFGB_MAXN], acc_rc[NW][FFGB_MAXN * FFGB_MAXN];
  __shared__ double2 vsh[NW][FFGB_MAXN + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nn = norb * norb;
  for (int i = lane; i < nn; i += 32) {
    acc_rr[warp][i] = make_double2(0.0, 0.0);
    acc_rc[warp][i] = make_double2(0.0, 0.0);
  }
  const int r = blockIdx.x * PAIR_ROWS + warp;
  if (r < rows) {
    const Cx* xr = x + (long long)r * cols;
    const Cx* yr = y + (long long)r * cols;
    Cx tot, cj[FFGB_MAXN];
    tot.x = tot.y = (T)0;
#pragma unroll
    for (int j = 0; j < FFGB_MAXN; ++j) cj[j].x = cj[j].y = (T)0;
    for (int c = lane; c < cols; c += 32) {
      Cx w;
      w.x = w.y = (T)0;
      w = cdot_row(w, xr[c], yr[c]);
      tot.x += w.x;
      tot.y += w.y;
      const unsigned sc = cstr[c];
#pragma unroll
      for (int j = 0; j < FFGB_MAXN; ++j)
        if ((sc >> j) & 1u) {
          cj[j].x += w.x;
          cj[j].y += w.y;
        }
    }
    // butterfly sums in FP64: every lane ends with the row's totals
    double2 R = to_d2(tot);
    for (int o = 16; o > 0; o >>= 1) {
      R.x += __shfl_xor_sync(0xffffffffu, R.x, o);
      R.y += __shfl_xor_sync(0xffffffffu, R.y, o);
    }
#pragma unroll
    for (int j = 0; j < FFGB_MAXN; ++j) {
      if (j < norb) {  // uniform
        double2 v = to_d2(cj[j]);
        for (int o = 16; o > 0; o >>= 1) {
          v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
          v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (lane == 0) vsh[warp][j] = v;
      }
    }
    __syncwarp();
    const unsigned sr = rstr[r];
    for (int idx = lane; idx < nn; idx += 32) {
      const int i = idx / norb, j = idx - i * norb;
      if (!((sr >> i) & 1u)) continue;
      const double2 v = vsh[warp][j];
      acc_rc[warp][idx].x += v.x;
      acc_rc[warp][idx].y += v.y;
      if ((sr >> j) & 1u) {
        acc_rr[warp][idx].x += R.x;
        acc_rr[warp][idx].y += R.y;
      }
    }
  }
  __syncthreads();
  double2* out = partial + (long long)blockIdx.x * 2 * nn;
  for (int idx = threadIdx.x; idx < nn; idx += PAIR_THREADS) {
    double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
    for (int w = 0; w < NW; ++w) {
      a.x += acc_rr[w][idx].x;
      a.y += acc_rr[w][idx].y;
      b.x += acc_rc[w][idx].x;
      b.y += acc_rc[w][idx].y;
    }
    out[idx] = a;
    out[nn + idx] = b;
  }
}

// out[k] = sum over c < chunks of partial[c * per + k] in a fixed order: a
// CTA takes 32 consecutive k (coalesced 512-byte rows) and 32 interleaved
// subsets of c (c = g, g + 32, ...), each summed in order of c, then the 32
// subset sums in order of g.
constexpr int SUMB_K = 32, SUMB_G = 32;
__global__ void __launch_bounds__(SUMB_K * SUMB_G) sum_blocks_kernel(const double2* __restrict__ partial,
                                                                     long long chunks, int per,
                                                                     double2* __restrict__ out) {
  __shared__ double2 sh[SUMB_G][SUMB_K + 1];
  const int kl = threadIdx.x % SUMB_K, g = threadIdx.x / SUMB_K;
  const int k = blockIdx.x * SUMB_K + kl;
  double2 a = make_double2(0.0, 0.0);
  if (k < per) {
#pragma unroll 4
    for (long long c = g; c < chunks; c += SUMB_G) {
      const double2 v = partial[c * per + k];
      a.x += v.x;
      a.y += v.y;
    }
  }
  sh[g][kl] = a;
  __syncthreads();
  if (g == 0 && k < per) {
    double2 t = sh[0][kl];
    for (int j = 1; j < SUMB_G; ++j) {
      t.x += sh[j][kl].x;
      t.y += sh[j][kl].y;
    }
    out[k] = t;
  }
}

// out[k] = sum over c < chunks of partial[k * chunks + c]: one warp per k,
// lanes over c (in order within a lane), then a fixed shuffle tree.
__global__ void __launch_bounds__(256) sum_chunks_kernel(const double2* __restrict__ partial, int chunks, int n,
                                                         double2* __restrict__ out) {
  const int k = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= n) return;
  double2 a = make_double2(0.0, 0.0);
  for (int c = lane; c < chunks; c += 32) {
    const double2 v = partial[(long long)k * chunks + c];
    a.x += v.x;
    a.y += v.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    a.x += __shfl_down_sync(0xffffffffu, a.x, o);
    a.y += __shfl_down_sync(0xffffffffu, a.y, o);
  }
  if (lane == 0) out[k] = a;
}

}  // namespace

// Transition one-body density of the sector on the rows of x, y (rows x cols)
// into g_dev (norb * norb complex, device memory), without synchronizing.
// complex64 sectors with 1 <= nocc and at most 10 vacancies per (nocc-1)-string
// run rdm1_sub_kernel (large) or rdm1_small_kernel over `sub` (the nocc-1
// strings); others rdm1_kernel, whose partials sum_chunks_kernel reduces.
template <typename T>
int rdm1_rows_dev(const void* x, const void* y, const unsigned* strings, int rows, int cols, int norb,
                  void* partial_buf, size_t partial_bytes, double2* g_dev, cudaStream_t st, int nocc,
                  const unsigned* sub, int n_sub) {
  const int nv = norb - nocc + 1;
  // large sectors: rdm1_sub_kernel (registers hold a third of the block per
  // thread, columns split over the CTA); small ones, whose states sit in L2:
  // rdm1_small_kernel (a warp per block entry)
  const bool large = (long long)rows * cols >= (1LL << 23);
  if (norb <= 0) return FFGB_OK;
  if (sizeof(T) == 4 && sub && nocc >= 1 && nv >= 1 && nv <= 10 && n_sub > 0 && cols > 0) {
    const size_t need = sizeof(double2) * (size_t)n_sub * nv * nv;
    if (need > partial_bytes) return fail(FFGB_ERR_OOM, "scratch too small for density partial sums");
    double2* part = (double2*)partial_buf;
    switch (nv) {
      case 1: return launch_rdm1_sub<1>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      case 2: return launch_rdm1_sub<2>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      case 3: return launch_rdm1_sub<3>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      case 4: return launch_rdm1_sub<4>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      case 5: return launch_rdm1_sub<5>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      case 6: return launch_rdm1_sub<6>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      case 7: return launch_rdm1_sub<7>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      case 8: return launch_rdm1_sub<8>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      case 9: return launch_rdm1_sub<9>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
      default: return launch_rdm1_sub<10>(x, y, sub, n_sub, cols, norb, part, g_dev, !large, st);
    }
  }
  const int chunks = (rows + RDM_ROWS - 1) / RDM_ROWS;
  const size_t need = sizeof(double2) * (size_t)chunks * norb * norb;
  if (need > partial_bytes) return fail(FFGB_ERR_OOM, "scratch too small for density partial sums");
  if (rows <= 0 || cols <= 0) {
    FFGB_CUDA(cudaMemsetAsync(g_dev, 0, sizeof(double2) * (size_t)norb * norb, st));
    return FFGB_OK;
  }
  dim3 grid((unsigned)chunks, (unsigned)(norb * norb));
  rdm1_kernel<T><<<grid, DTHREADS, 0, st>>>((const typename CT<T>::type*)x, (const typename CT<T>::type*)y,
                                            strings, rows, cols, norb, (double2*)partial_buf);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  sum_chunks_kernel<<<(unsigned)((norb * norb + 7) / 8), 256, 0, st>>>((const double2*)partial_buf, chunks,
                                                                      norb * norb, g_dev);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

// The same, read back to the host (synchronizes).
template <typename T>
int rdm1_rows(const void* x, const void* y, const unsigned* strings, int rows, int cols, int norb,
              void* partial_buf, size_t partial_bytes, std::vector<double>& out, cudaStream_t st, int nocc,
              const unsigned* sub, int n_sub) {
  const size_t n2 = (size_t)norb * norb;
  if (partial_bytes < sizeof(double2) * n2 + 256) return fail(FFGB_ERR_OOM, "scratch too small for densities");
  // the result at the end of the partial buffer
  const size_t tail = (partial_bytes - sizeof(double2) * n2) / 256 * 256;
  double2* g = (double2*)((char*)partial_buf + tail);
  FFGB_TRY(rdm1_rows_dev<T>(x, y, strings, rows, cols, norb, partial_buf, tail, g, st, nocc, sub, n_sub));
  out.assign(2 * n2, 0.0);
  if (n2) {
    FFGB_CUDA(cudaMemcpyAsync(out.data(), g, sizeof(double2) * n2, cudaMemcpyDeviceToHost, st));
    FFGB_CUDA(cudaStreamSynchronize(st));
  }
  return FFGB_OK;
}

// Pair densities (row-row and row-column) of x, y with rows indexed by rstr
// into sums_dev (2 * norb * norb complex: row-row, then row-column), without
// synchronizing.
template <typename T>
int pair_rows_dev(const void* x, const void* y, const unsigned* rstr, const unsigned* cstr, int rows, int cols,
                  int norb, void* partial_buf, size_t partial_bytes, double2* sums_dev, cudaStream_t st) {
  const long long chunks = (rows + PAIR_ROWS - 1) / PAIR_ROWS;
  const int per = 2 * norb * norb;
  const size_t need = sizeof(double2) * (size_t)chunks * per;
  if (need > partial_bytes) return fail(FFGB_ERR_OOM, "scratch too small for density partial sums");
  if (per == 0) return FFGB_OK;
  if (rows <= 0 || cols <= 0) {
    FFGB_CUDA(cudaMemsetAsync(sums_dev, 0, sizeof(double2) * per, st));
    return FFGB_OK;
  }
  double2* part = (double2*)partial_buf;
  pair_density_kernel<T><<<(unsigned)chunks, PAIR_THREADS, 0, st>>>((const typename CT<T>::type*)x,
                                                                    (const typename CT<T>::type*)y, rstr, cstr,
                                                                    rows, cols, norb, part);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  sum_blocks_kernel<<<(per + SUMB_K - 1) / SUMB_K, SUMB_K * SUMB_G, 0, st>>>(part, chunks, per, sums_dev);
  count_launch();
  FFGB_CUDA(cudaGetLastError());
  return FFGB_OK;
}

// The same, read back to the host (synchronizes).
template <typename T>
int pair_rows(const void* x, const void* y, const unsigned* rstr, const unsigned* cstr, int rows, int cols,
              int norb, void* partial_buf, size_t partial_bytes, std::vector<double>& rr, std::vector<double>& rc,
              cudaStream_t st) {
  const size_t per = 2 * (size_t)norb * norb;
  if (partial_bytes < sizeof(double2) * per + 256) return fail(FFGB_ERR_OOM, "scratch too small for densities");
  const size_t tail = (partial_bytes - sizeof(double2) * per) / 256 * 256;
  double2* sums = (double2*)((char*)partial_buf + tail);
  FFGB_TRY(pair_rows_dev<T>(x, y, rstr, cstr, rows, cols, norb, partial_buf, tail, sums, st));
  rr.assign(2 * (size_t)norb * norb, 0.0);
  rc.assign(2 * (size_t)norb * norb, 0.0);
  if (!per) return FFGB_OK;
  std::vector<double> h(2 * per, 0.0);
  FFGB_CUDA(cudaMemcpyAsync(h.data(), sums, sizeof(double2) * per, cudaMemcpyDeviceToHost, st));
  FFGB_CUDA(cudaStreamSynchronize(st));
  std::memcpy(rr.data(), h.data(), sizeof(double) * 2 * norb * norb);
  std::memcpy(rc.data(), h.data() + 2 * (size_t)norb * norb, sizeof(double) * 2 * norb * norb);
  return FFGB_OK;
}

template int rdm1_rows<float>(const void*, const void*, const unsigned*, int, int, int, void*, size_t,
                              std::vector<double>&, cudaStream_t, int, const unsigned*, int);
template int rdm1_rows<double>(const void*, const void*, const unsigned*, int, int, int, void*, size_t,
                               std::vector<double>&, cudaStream_t, int, const unsigned*, int);
template int pair_rows<float>(const void*, const void*, const unsigned*, const unsigned*, int, int, int, void*,
                              size_t, std::vector<double>&, std::vector<double>&, cudaStream_t);
template int pair_rows<double>(const void*, const void*, const unsigned*, const unsigned*, int, int, int, void*,
                               size_t, std::vector<double>&, std::vector<double>&, cudaStream_t);
template int rdm1_rows_dev<float>(const void*, const void*, const unsigned*, int, int, int, void*, size_t,
                                  double2*, cudaStream_t, int, const unsigned*, int);
template int rdm1_rows_dev<double>(const void*, const void*, const unsigned*, int, int, int, void*, size_t,
                                   double2*, cudaStream_t, int, const unsigned*, int);
template int pair_rows_dev<float>(const void*, const void*, const unsigned*, const unsigned*, int, int, int,
                                  void*, size_t, double2*, cudaStream_t);
template int pair_rows_dev<double>(const void*, const void*, const unsigned*, const unsigned*, int, int, int,
                                   void*, size_t, double2*, cudaStream_t);

// Partial-sum bytes the density kernels need for a sector of `rows` strings
// (also enough for rdm1_sub_kernel's blocks: at most rows * norb * ... see below).
size_t density_partial_bytes(int norb, long long rows) {
  const long long chunks = std::max((rows + RDM_ROWS - 1) / RDM_ROWS, (rows + PAIR_ROWS - 1) / PAIR_ROWS);
  return sizeof(double2) * ((size_t)chunks + 1) * 2 * norb * norb + 256;
}

// Partial-sum bytes of rdm1_sub_kernel for n_sub strings with nv vacancies.
size_t density_sub_bytes(int norb, long long n_sub, int nv) {
  return sizeof(double2) * ((size_t)n_sub * nv * nv + (size_t)norb * norb) + 256;
}

}  // namespace ffgb
