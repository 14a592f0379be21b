// Device code of the sector kernels.
//
// A *pass* processes a 2-D array whose rows are complete state vectors of
// one spin sector (the *rotated* sector, `dim` = C(norb, nocc) entries per
// row) while the row index enumerates the strings of the other sector.  A
// CTA stages `rows_per_cta` consecutive rows in shared memory, applies the
// orbital-rotation plan of the rotated sector to every row, then runs the
// epilogue: optional final orbital phases, optional diagonal operator
// (phase exp(i f) or real coefficient f), and an output mode (store in the
// same layout, store transposed, accumulate, or reduce sum f |v|^2).
//
// Storing transposed lets two passes rotate both spin sectors of a
// (dim_a, dim_b) state with only row-contiguous reads: pass A rotates the
// beta sector of each alpha row and writes the (dim_b, dim_a) transpose;
// pass B rotates the alpha sector of each beta row and writes back.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#define FFGB_MAXN 18
#define FFGB_MAXTRI (FFGB_MAXN * (FFGB_MAXN - 1) / 2)
#define FFGB_BST (FFGB_MAXN + 2)  // stride of the binomial table

namespace ffgb {

enum { OUT_STORE = 0, OUT_ACCUM = 1, OUT_EXPECT = 2, OUT_NONE = 3 };
enum { LAYOUT_SAME = 0, LAYOUT_T = 1 };
enum { DIAG_NONE = 0, DIAG_PHASE = 1, DIAG_COEF = 2 };
enum { KIND_IDENTITY = 0, KIND_TRIANGLE = 1, KIND_FULL = 2, KIND_CSD = 3 };

template <typename T>
struct CT;
template <>
struct CT<float> {
  using type = float2;
};
template <>
struct CT<double> {
  using type = double2;
};

template <typename T>
struct SectorParams {
  // rotated sector and its plan
  int norb, nocc, dim;
  int kind, h, n_tri;
  T tri[FFGB_MAXTRI * 3];
  signed char tri_l[FFGB_MAXTRI];
  T win[4][28 * 3];
  T cs[8][8];
  int comp;              // apply the FP32 rounding residuals of the window/CS coefficients
  T win_lo[4][28 * 3];
  T cs_lo[8][8];
  int has_dphase;
  T dphase[FFGB_MAXN][2];
  // rows
  long long n_rows;
  int rows_per_cta;
  int row_norb, row_nocc;
  const unsigned* row_strings;
  const unsigned* col_strings;
  // io
  const void* in;
  void* out;
  int out_op, layout;
  T alpha_re, alpha_im;
  // diagonal operator f(r, j) = F_R(r) + F_C(j) + sum_{i,l} cross[i][l] g_i(r) g_l(j)
  int diag_mode, zrep;
  double rsame[FFGB_MAXN][FFGB_MAXN];
  double cross[FFGB_MAXN][FFGB_MAXN];
  const void* col_table;
  double* partials;
  int chunk_bits;
};

struct Layout {
  int binom, plan, tab, dt, xt, red, rows, total;
  int nch, chunk_bits, dch;
};

__host__ __device__ inline int align16(int x) { return (x + 15) & ~15; }

// Shared-memory layout; identical on host and device.
__host__ __device__ inline Layout make_layout(int tsize, int R, int dim, int col_norb,
                                              int chunk_bits, int has_dphase, int diag_mode,
                                              int kind, int comp) {
  Layout L;
  int off = 0;
  L.binom = off;
  off += align16(FFGB_BST * FFGB_BST * 4);
  L.plan = off;
  if (kind == KIND_TRIANGLE) off += align16(FFGB_MAXTRI * 3 * tsize);
  if (kind == KIND_FULL || kind == KIND_CSD) off += align16((comp ? 2 : 1) * (4 * 28 * 3 + 64) * tsize);
  L.tab = off;
  off += align16(256 * 2 + 256 * 4 + 16 * 4);
  // cross-half pair table: (k, i) -> packed (j, jp, parity) entries and offsets
  if (kind == KIND_CSD) off += align16(1024 * 2 + 9 * 8 * 2 + 16);
  if (kind == KIND_CSD || kind == KIND_FULL) off += align16(72 * 4);  // identity member offsets
  L.chunk_bits = chunk_bits;
  L.nch = (col_norb + chunk_bits - 1) / chunk_bits;
  if (L.nch < 1) L.nch = 1;
  const int nent = L.nch << chunk_bits;
  // final orbital phases: 4-bit chunks (small table, a few more multiplies)
  L.dch = (col_norb + 3) / 4;
  if (L.dch < 1) L.dch = 1;
  L.dt = off;
  if (has_dphase && diag_mode != DIAG_PHASE) off += align16((L.dch << 4) * 2 * tsize);
  L.xt = off;
  if (diag_mode == DIAG_PHASE) off += align16(nent * 2 * tsize + 2 * FFGB_MAXN * 8 + 16);
  if (diag_mode == DIAG_COEF) off += align16(nent * tsize + 2 * FFGB_MAXN * 8 + 16);
  L.red = off;
  off += align16(33 * 8);
  L.rows = off;
  off += align16(R * dim * 2 * tsize);
  L.total = off;
  return L;
}

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <typename C>
__device__ __forceinline__ C cmake(double re, double im);
template <>
__device__ __forceinline__ float2 cmake<float2>(double re, double im) {
  return make_float2((float)re, (float)im);
}
template <>
__device__ __forceinline__ double2 cmake<double2>(double re, double im) {
  return make_double2(re, im);
}

// exp(i theta) with theta in FP64, rounded once to the output type.
__device__ __forceinline__ float2 phase_of(double theta, float2*) {
  const double two_pi = 6.283185307179586476925286766559;
  double r = theta - two_pi * rint(theta * 0.15915494309189533576888376337251);
  float hi = (float)r;
  float lo = (float)(r - (double)hi);
  float s, c;
  sincosf(hi, &s, &c);
  return make_float2(c - s * lo, s + c * lo);
}
__device__ __forceinline__ double2 phase_of(double theta, double2*) {
  double s, c;
  sincos(theta, &s, &c);
  return make_double2(c, s);
}

__device__ __forceinline__ int bn(const int* sB, int a, int b) {
  return (b < 0 || a < 0 || b > a) ? 0 : sB[a * FFGB_BST + b];
}

// colexicographic unranking of a k-subset of nbits
__device__ __forceinline__ unsigned unrank_colex(int t, int nbits, int k, const int* sB) {
  unsigned s = 0;
  for (int p = nbits - 1; p >= 0 && k > 0; --p) {
    int c = bn(sB, p, k);
    if (t >= c) {
      s |= 1u << p;
      t -= c;
      --k;
    }
  }
  return s;
}

// colexicographic rank = address among strings with the same popcount
__device__ __forceinline__ int rank_colex(unsigned s, const int* sB) {
  int r = 0, t = 0;
  while (s) {
    int p = __ffs(s) - 1;
    s &= s - 1;
    ++t;
    r += bn(sB, p, t);
  }
  return r;
}

// rank contribution of bits of s placed at orbital offset `base_orb` with
// `m0` electrons below them
__device__ __forceinline__ int rank_shifted(unsigned s, int base_orb, int m0, const int* sB) {
  int r = 0, t = m0;
  while (s) {
    int p = __ffs(s) - 1;
    s &= s - 1;
    ++t;
    r += bn(sB, base_orb + p, t);
  }
  return r;
}

// rotation of a complex64 pair by [[c, s], [-conj(s), c]]:
// x <- c x + s y, y <- -conj(s) x + c y, on packed FP32x2 (re, im) lanes.
// With COMP the coefficients are (c + cl, s + sl): the FP32 rounding residuals
// of the FP64 plan are applied first, so the rotation angle is exact to ~1e-14
// instead of ~6e-8.
template <bool COMP>
__device__ __forceinline__ void rot_pair(float2& x, float2& y, float c, float sr, float si, float cl,
                                         float srl, float sil) {
  const float2 xs = make_float2(x.y, x.x), ys = make_float2(y.y, y.x);
  const float2 i2 = make_float2(-si, si);
  float2 nx, ny;
  if constexpr (!COMP) {
    nx = __fmul2_rn(make_float2(c, c), x);
    ny = __fmul2_rn(make_float2(c, c), y);
  } else {
    const float2 il = make_float2(-sil, sil);
    nx = __fmul2_rn(make_float2(cl, cl), x);
    nx = __ffma2_rn(make_float2(srl, srl), y, nx);
    nx = __ffma2_rn(il, ys, nx);
    ny = __fmul2_rn(make_float2(cl, cl), y);
    ny = __ffma2_rn(make_float2(-srl, -srl), x, ny);
    ny = __ffma2_rn(il, xs, ny);
    nx = __ffma2_rn(make_float2(c, c), x, nx);
    ny = __ffma2_rn(make_float2(c, c), y, ny);
  }
  nx = __ffma2_rn(make_float2(sr, sr), y, nx);
  nx = __ffma2_rn(i2, ys, nx);
  ny = __ffma2_rn(make_float2(-sr, -sr), x, ny);
  ny = __ffma2_rn(i2, xs, ny);
  x = nx;
  y = ny;
}

// Coefficients (c, Re s, Im s) of rotation g of a window network.
//   MODE 0: FP32 values gp.
//   MODE 1: FP32 values gp plus FP32 residuals gl (compensated, see rot_pair).
//   MODE 2: dithered rounding.  gp / gl hold the two FP32 neighbours below /
//           above each FP64 coefficient and gt the probability of the upper
//           one as a 32-bit threshold.  Every thread draws its own choice from
//           its generator `rng`, so each column sees an unbiased rounding of
//           the plan and the rounding errors of different columns are
//           independent instead of identical.
template <int MODE>
__device__ __forceinline__ void win_coef(const float* __restrict__ gp, const float* __restrict__ gl,
                                         const unsigned* __restrict__ gt, int g, unsigned& rng, float& c,
                                         float& sr, float& si, float& cl, float& srl, float& sil) {
  if constexpr (MODE == 2) {
    float v[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      rng = rng * 1664525u + 1013904223u;
      v[q] = rng < gt[3 * g + q] ? gl[3 * g + q] : gp[3 * g + q];
    }
    c = v[0];
    sr = v[1];
    si = v[2];
    cl = srl = sil = 0.f;
  } else {
    c = gp[3 * g];
    sr = gp[3 * g + 1];
    si = gp[3 * g + 2];
    cl = MODE == 1 ? gl[3 * g] : 0.f;
    srl = MODE == 1 ? gl[3 * g + 1] : 0.f;
    sil = MODE == 1 ? gl[3 * g + 2] : 0.f;
  }
}

// Coefficients of one rotation for complement-packed members (split
// re / im lanes): c2 = (c, c), sa = (sr, -sr), sb = (-sr, sr),
// sip = (si, si), sim = (-si, -si).
struct PackCoef {
  float2 c2, sa, sb, sip, sim;
};

template <int MODE>
__device__ __forceinline__ void pack_coef(const float* __restrict__ gp, const float* __restrict__ gl,
                                          const unsigned* __restrict__ gt, int g, unsigned& rng, PackCoef& k) {
  float c, sr, si, cl, srl, sil;
  win_coef<MODE == 1 ? 0 : MODE>(gp, gl, gt, g, rng, c, sr, si, cl, srl, sil);
  k.c2 = make_float2(c, c);
  k.sa = make_float2(sr, -sr);
  k.sb = make_float2(-sr, sr);
  k.sip = make_float2(si, si);
  k.sim = make_float2(-si, -si);
}

// One rotation on two packs P, Q whose lanes are partners lane by lane:
// P <- c P + vp (.) Q, Q <- c Q + vq (.) P, with vp, vq = (s, -conj s) when
// VP_A / VQ_A, else (-conj s, s); complex lane products in split form.
template <bool VP_A, bool VQ_A>
__device__ __forceinline__ void rot_pack(float2& PR, float2& PI, float2& QR, float2& QI, const PackCoef& k) {
  const float2 rp = VP_A ? k.sa : k.sb, rq = VQ_A ? k.sa : k.sb;
  float2 pr = __fmul2_rn(k.c2, PR), pi = __fmul2_rn(k.c2, PI);
  float2 qr = __fmul2_rn(k.c2, QR), qi = __fmul2_rn(k.c2, QI);
  pr = __ffma2_rn(rp, QR, pr);
  pr = __ffma2_rn(k.sim, QI, pr);
  pi = __ffma2_rn(rp, QI, pi);
  pi = __ffma2_rn(k.sip, QR, pi);
  qr = __ffma2_rn(rq, PR, qr);
  qr = __ffma2_rn(k.sim, PI, qr);
  qi = __ffma2_rn(rq, PI, qi);
  qi = __ffma2_rn(k.sip, PR, qi);
  PR = pr;
  PI = pi;
  QR = qr;
  QI = qi;
}

// The same with lane 0 of P partnering lane 1 of Q (and lane 1 of P lane 0 of Q).
template <bool VP_A, bool VQ_A>
__device__ __forceinline__ void rot_pack_x(float2& PR, float2& PI, float2& QR, float2& QI, const PackCoef& k) {
  const float2 rp = VP_A ? k.sa : k.sb, rq = VQ_A ? k.sa : k.sb;
  const float2 QRs = make_float2(QR.y, QR.x), QIs = make_float2(QI.y, QI.x);
  const float2 PRs = make_float2(PR.y, PR.x), PIs = make_float2(PI.y, PI.x);
  float2 pr = __fmul2_rn(k.c2, PR), pi = __fmul2_rn(k.c2, PI);
  float2 qr = __fmul2_rn(k.c2, QR), qi = __fmul2_rn(k.c2, QI);
  pr = __ffma2_rn(rp, QRs, pr);
  pr = __ffma2_rn(k.sim, QIs, pr);
  pi = __ffma2_rn(rp, QIs, pi);
  pi = __ffma2_rn(k.sip, QRs, pi);
  qr = __ffma2_rn(rq, PRs, qr);
  qr = __ffma2_rn(k.sim, PIs, qr);
  qi = __ffma2_rn(rq, PIs, qi);
  qi = __ffma2_rn(k.sip, PRs, qi);
  PR = pr;
  PI = pi;
  QR = qr;
  QI = qi;
}

// Start of a thread's generator for dithered coefficients (a hash of the
// column and the stage's salt).
__device__ __forceinline__ unsigned dither_seed(unsigned long long col, unsigned salt) {
  unsigned x = (unsigned)col * 0x9E3779B9u ^ (unsigned)(col >> 32) ^ salt;
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

}  // namespace ffgb

namespace ffgb {
// The two halves of rot_pair, for a pair whose members sit in different
// threads: x <- c x + s y (the thread holding x) and y <- -conj(s) x + c y
// (the thread holding y), with the same operations and rounding as rot_pair
// with plain or dithered coefficients.
__device__ __forceinline__ void rot_half_x(float2& x, float2 y, float c, float sr, float si) {
  const float2 ys = make_float2(y.y, y.x);
  float2 nx = __fmul2_rn(make_float2(c, c), x);
  nx = __ffma2_rn(make_float2(sr, sr), y, nx);
  nx = __ffma2_rn(make_float2(-si, si), ys, nx);
  x = nx;
}
__device__ __forceinline__ void rot_half_y(float2& y, float2 x, float c, float sr, float si) {
  const float2 xs = make_float2(x.y, x.x);
  float2 ny = __fmul2_rn(make_float2(c, c), y);
  ny = __ffma2_rn(make_float2(-sr, -sr), x, ny);
  ny = __ffma2_rn(make_float2(-si, si), xs, ny);
  y = ny;
}

#include "windows_gen.cuh"
}

namespace ffgb {

// Distribute work items to warps so that each warp handles 32 items of one
// class k (the register-array shape depends on k).  Classes run from the
// middle of [kbeg, kend] outwards (largest groups first) and consecutive
// tasks go to consecutive warps, so few distinct code paths are live at once.
template <class CountF, class Body>
__device__ __forceinline__ void warp_tasks(int kbeg, int kend, CountF count, Body body) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int kmid = (kbeg + kend) >> 1;
  int t0 = 0;
  for (int step = 0; step <= kend - kbeg; ++step) {
    const int k = (step & 1) ? kmid + ((step + 1) >> 1) : kmid - (step >> 1);
    if (k < kbeg || k > kend) continue;
    const int n = count(k);
    const int nt = (n + 31) >> 5;
    int first = warp - (t0 % nw);
    if (first < 0) first += nw;
    for (int t = first; t < nt; t += nw) {
      const int item = t * 32 + lane;
      if (item < n) body(k, item);
    }
    t0 += nt;
  }
}

// ---------------------------------------------------------------------------
// the sector kernel
// ---------------------------------------------------------------------------

__device__ __forceinline__ void cp_async8(void* s, const void* g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async16(void* s, const void* g) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(s);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Copy `bytes` (a multiple of 8) from global to shared memory with the
// asynchronous copy unit; 16-byte copies when both sides allow it.
__device__ __forceinline__ void stage_rows(void* dst, const void* src, long long bytes) {
  const int tid = threadIdx.x, nth = blockDim.x;
  if ((((uintptr_t)dst | (uintptr_t)src) & 15) == 0 && (bytes & 15) == 0) {
    const long long n = bytes >> 4;
    for (long long i = tid; i < n; i += nth)
      cp_async16((char*)dst + (i << 4), (const char*)src + (i << 4));
  } else {
    const long long n = bytes >> 3;
    for (long long i = tid; i < n; i += nth) cp_async8((char*)dst + (i << 3), (const char*)src + (i << 3));
  }
  cp_async_wait_all();
}

// Persistent CTAs: each CTA builds its tables once and then processes the row
// chunks blockIdx.x, blockIdx.x + gridDim.x, ...
// Threads per CTA of the sector kernel: windows of 8 orbitals hold 70
// complex64 members per thread, so those kernels run 128 threads with the
// full register file share of 2 CTAs per SM.
__host__ __device__ constexpr int sector_threads(int nw) {
  return nw == 0 ? 256 : ((nw == 8 || nw >= 15) ? 128 : 192);
}

template <typename T, int NW>
__global__ void __launch_bounds__(sector_threads(NW), NW > 0 ? 2 : 1)
    sector_kernel(const __grid_constant__ SectorParams<T> P) {
  using C = typename CT<T>::type;
  extern __shared__ __align__(16) unsigned char smem[];
  const Layout L = make_layout((int)sizeof(T), P.rows_per_cta, P.dim, P.norb, P.chunk_bits,
                               P.has_dphase, P.diag_mode, P.kind, P.comp);
  // final orbital phases are folded into the per-row phase tables when both are present
  const bool sep_dphase = P.has_dphase && P.diag_mode != DIAG_PHASE;
  int* sB = (int*)(smem + L.binom);
  T* sPlan = (T*)(smem + L.plan);
  unsigned short* sS2 = (unsigned short*)(smem + L.tab);
  int* sRT = (int*)(smem + L.tab + 512);
  int* sMoff = (int*)(smem + L.tab + 512 + 1024);
  C* srow = (C*)(smem + L.rows);
  double* sRed = (double*)(smem + L.red);

  const int tid = threadIdx.x, nth = blockDim.x;
  const int dim = P.dim, norb = P.norb, nocc = P.nocc;
  const long long n_chunks = (P.n_rows + P.rows_per_cta - 1) / P.rows_per_cta;

  // ------------------------------------------------------------ per-CTA setup
  for (int idx = tid; idx < FFGB_BST * FFGB_BST; idx += nth) {
    const int a = idx / FFGB_BST, b = idx % FFGB_BST;
    int v = 0;
    if (b <= a) {
      int r = 1;
      for (int i = 1; i <= b; ++i) r = r * (a - b + i) / i;  // exact: r * (a-b+i) is divisible by i
      v = r;
    }
    sB[idx] = v;
  }
  if (P.kind == KIND_TRIANGLE) {
    for (int idx = tid; idx < P.n_tri * 3; idx += nth) sPlan[idx] = P.tri[idx];
  } else if (P.kind == KIND_FULL || P.kind == KIND_CSD) {
    for (int idx = tid; idx < 4 * 28 * 3; idx += nth) sPlan[idx] = (&P.win[0][0])[idx];
    for (int idx = tid; idx < 64; idx += nth) sPlan[4 * 28 * 3 + idx] = (&P.cs[0][0])[idx];
    int* sId = (int*)(smem + L.tab + (P.kind == KIND_CSD ? align16(1600 + 1024 * 2 + 9 * 8 * 2 + 16) : 1600));
    for (int idx = tid; idx < 72; idx += nth) sId[idx] = idx;
    if (P.comp) {
      for (int idx = tid; idx < 4 * 28 * 3; idx += nth) sPlan[400 + idx] = (&P.win_lo[0][0])[idx];
      for (int idx = tid; idx < 64; idx += nth) sPlan[400 + 4 * 28 * 3 + idx] = (&P.cs_lo[0][0])[idx];
    }
  }
  constexpr int H = (NW <= 8) ? NW : NW / 2;
  constexpr int Q = NW - H;
  if constexpr (NW > 8) {
    __syncthreads();
    if (tid <= Q) {
      int o = 0;
      for (int m = 0; m < tid; ++m) o += bn(sB, Q, m);
      sMoff[tid] = o;
    }
    __syncthreads();
    for (int idx = tid; idx < (1 << Q); idx += nth) {
      int m = 0;
      while (m < Q && idx >= sMoff[m + 1]) ++m;
      const int g = idx - sMoff[m];
      const unsigned s2 = unrank_colex(g, Q, m, sB);
      sS2[idx] = (unsigned short)s2;
      const int m0 = nocc - m;
      sRT[idx] = (m0 >= 0 && m0 <= H) ? rank_shifted(s2, H, m0, sB) : 0;
    }
    // pair table of the cross-half rotations: for k electrons in the low half
    // and site i, every member j (colex index) of the k-family with bit i set,
    // the index jp of its partner (bit i cleared) in the (k-1)-family and the
    // parity of the low-half orbitals occupied above i.
    unsigned short* sCS = (unsigned short*)(smem + L.tab + 1600);
    unsigned short* sCSo = sCS + 1024;  // [k][i] offsets, k in 1..H
    if (tid == 0) {
      int o = 0;
      for (int k = 1; k <= H; ++k)
        for (int i = 0; i < H; ++i) {
          sCSo[(k - 1) * 8 + i] = (unsigned short)o;
          o += bn(sB, H - 1, k - 1);
        }
    }
    __syncthreads();
    if (tid < H * H) {  // one thread per (k, i) fills its list
      const int k = tid / H + 1, i = tid % H;
      unsigned short* dst = sCS + sCSo[(k - 1) * 8 + i];
      const int nk = bn(sB, H, k);
      int pos = 0;
      for (int j = 0; j < nk; ++j) {
        const unsigned w = unrank_colex(j, H, k, sB);
        if (!((w >> i) & 1u)) continue;
        const int jp = rank_colex(w ^ (1u << i), sB);
        const int par = __popc(w >> (i + 1)) & 1;
        dst[pos++] = (unsigned short)(j | (jp << 7) | (par << 14));
      }
    }
  }
  const int cb = L.chunk_bits, nch = L.nch, nent = nch << cb;
  const unsigned cmask = (1u << cb) - 1u;
  C* sDT = (C*)(smem + L.dt);
  const int dch = L.dch;
  if (sep_dphase) {
    for (int e = tid; e < (dch << 4); e += nth) {
      const int c = e >> 4;
      unsigned x = (unsigned)(e & 15);
      C ph = cmake<C>(1.0, 0.0);
      while (x) {
        const int b = __ffs(x) - 1;
        x &= x - 1;
        const int orb = c * 4 + b;
        if (orb < norb) {
          C d;
          d.x = P.dphase[orb][0];
          d.y = P.dphase[orb][1];
          ph = cmul(ph, d);
        }
      }
      sDT[e] = ph;
    }
  }
  C* sXP = (C*)(smem + L.xt);
  T* sXC = (T*)(smem + L.xt);
  double* sM = (double*)(smem + L.xt + (P.diag_mode == DIAG_PHASE ? align16(nent * 2 * (int)sizeof(T))
                                                                   : align16(nent * (int)sizeof(T))));
  const C* colP = (const C*)P.col_table;
  const T* colZ = (const T*)P.col_table;
  C* out = (C*)P.out;
  double acc_d = 0.0;
  float acc_f = 0.f, comp_f = 0.f;
  __syncthreads();

  for (long long chunk = blockIdx.x; chunk < n_chunks; chunk += gridDim.x) {
    const long long row0 = chunk * P.rows_per_cta;
    const long long rem = P.n_rows - row0;
    const int R = (int)(rem < P.rows_per_cta ? rem : P.rows_per_cta);

    // rows [row0, row0 + R) are contiguous in the input
    stage_rows(srow, (const C*)P.in + row0 * (long long)dim, (long long)R * dim * (long long)sizeof(C));
    __syncthreads();

    // ------------------------------------------------------------- stages
    if constexpr (NW == 0) {
      if (P.kind == KIND_TRIANGLE && nocc >= 1 && nocc <= norb - 1) {
        const int npairs = bn(sB, norb - 2, nocc - 1);
        const int items = R * npairs;
        for (int g = 0; g < P.n_tri; ++g) {
          const int l = P.tri_l[g];
          const T c = sPlan[3 * g], sr = sPlan[3 * g + 1], si = sPlan[3 * g + 2];
          const unsigned lowmask = (1u << l) - 1u;
          for (int item = tid; item < items; item += nth) {
            const int rho = item / npairs, t = item - rho * npairs;
            const unsigned p = unrank_colex(t, norb - 2, nocc - 1, sB);
            const unsigned x = (p & lowmask) | (1u << l) | ((p >> l) << (l + 2));
            const int rx = rank_colex(x, sB);
            const int ry = rx + bn(sB, l, __popc(p & lowmask));
            C* base = srow + (long long)rho * dim;
            const C a = base[rx], b = base[ry];
            C na, nb;
            na.x = c * a.x + sr * b.x - si * b.y;
            na.y = c * a.y + sr * b.y + si * b.x;
            nb.x = c * b.x - sr * a.x - si * a.y;
            nb.y = c * b.y - sr * a.y + si * a.x;
            base[rx] = na;
            base[ry] = nb;
          }
          __syncthreads();
        }
      }
    } else {
      static_assert(NW == 0 || sizeof(T) == 4, "window kernels are complex64 only");
      const float* wp = (const float*)sPlan;
      const int* sId = (const int*)(smem + L.tab + (NW > 8 ? align16(1600 + 1024 * 2 + 9 * 8 * 2 + 16) : 1600));
      if constexpr (NW <= 8) {
        // the whole sector is one window
        for (int rho = tid; rho < R; rho += nth) {
          if (P.comp)
            WinDispatch<H>::template group<true>(nocc, srow + (long long)rho * dim, sId, wp, wp + 400);
          else
            WinDispatch<H>::template group<false>(nocc, srow + (long long)rho * dim, sId, wp, wp);
        }
        __syncthreads();
      } else {
        const int klo_low = max(0, nocc - Q), khi_low = min(H, nocc);
        const int klo_high = max(0, nocc - H), khi_high = min(Q, nocc);
        auto low_stage = [&](const float* gp) {
          warp_tasks(
              klo_low, khi_low, [&](int k) { return R * bn(sB, Q, nocc - k); },
              [&](int k, int item) {
                const int G = bn(sB, Q, nocc - k);
                const int rho = item / G, g = item - rho * G;
                const int base = rho * dim + sRT[sMoff[nocc - k] + g];
                if (P.comp)
                  WinDispatch<H>::template group<true>(k, srow + base, sId, gp, gp + 400);
                else
                  WinDispatch<H>::template group<false>(k, srow + base, sId, gp, gp);
              });
          __syncthreads();
        };
        auto high_stage = [&](const float* gp) {
          warp_tasks(
              klo_high, khi_high, [&](int k) { return R * bn(sB, H, nocc - k); },
              [&](int k, int item) {
                const int G = bn(sB, H, nocc - k);
                const int rho = item / G, g = item - rho * G;
                if (P.comp)
                  WinDispatch<Q>::template group<true>(k, srow + rho * dim + g, sRT + sMoff[k], gp, gp + 400);
                else
                  WinDispatch<Q>::template group<false>(k, srow + rho * dim + g, sRT + sMoff[k], gp, gp);
              });
          __syncthreads();
        };
        low_stage(wp + 0 * 84);
        high_stage(wp + 1 * 84);
        // cross-half rotations (i, H + i): for each site, the groups of the
        // low-half window whose high part lacks bit i (s2 enumerated over the
        // other Q-1 high orbitals), each pair read from the shared table.
        const float* csp = wp + 4 * 84;
        const unsigned short* sCS = (const unsigned short*)(smem + L.tab + 1600);
        const unsigned short* sCSo = sCS + 1024;
        for (int i = 0; i < H; ++i) {
          const float g00r = csp[8 * i + 0], g00i = csp[8 * i + 1], g01r = csp[8 * i + 2],
                      g01i = csp[8 * i + 3], g10r = csp[8 * i + 4], g10i = csp[8 * i + 5],
                      g11r = csp[8 * i + 6], g11i = csp[8 * i + 7];
          const float* csl = csp + 400;
          const bool comp = P.comp != 0;
          const float l00r = comp ? csl[8 * i + 0] : 0.f, l00i = comp ? csl[8 * i + 1] : 0.f,
                      l01r = comp ? csl[8 * i + 2] : 0.f, l01i = comp ? csl[8 * i + 3] : 0.f,
                      l10r = comp ? csl[8 * i + 4] : 0.f, l10i = comp ? csl[8 * i + 5] : 0.f,
                      l11r = comp ? csl[8 * i + 6] : 0.f, l11i = comp ? csl[8 * i + 7] : 0.f;
          const unsigned lowm = (1u << i) - 1u;
          warp_tasks(
              max(1, klo_low), min(khi_low, nocc), [&](int k) { return R * bn(sB, Q - 1, nocc - k); },
              [&](int k, int item) {
                const int m = nocc - k;
                const int G = bn(sB, Q - 1, m);
                const int rho = item / G, g = item - rho * G;
                const unsigned s2r = unrank_colex(g, Q - 1, m, sB);
                const unsigned s2 = (s2r & lowm) | ((s2r >> i) << (i + 1));
                float2* bx = srow + rho * dim + rank_shifted(s2, H, k, sB);
                float2* by = srow + rho * dim + rank_shifted(s2 | (1u << i), H, k - 1, sB);
                const int sg0 = __popc(s2 & lowm) & 1;
                const unsigned short* tab = sCS + sCSo[(k - 1) * 8 + i];
                const int cnt = bn(sB, H - 1, k - 1);
                auto run = [&](auto comp_tag) {
                  constexpr bool CP = decltype(comp_tag)::value;
#pragma unroll 2
                  for (int t = 0; t < cnt; ++t) {
                    const unsigned e = tab[t];
                    const int j = e & 127, jp = (e >> 7) & 127;
                    const float sgn = (((e >> 14) ^ sg0) & 1) ? -1.f : 1.f;
                    const float2 x = bx[j], y = by[jp];
                    float ax = 0.f, ay = 0.f, bxr = 0.f, byi = 0.f;
                    if constexpr (CP) {  // FP32 rounding residuals of the coefficients first
                      ax = l00r * x.x - l00i * x.y + sgn * (l01r * y.x - l01i * y.y);
                      ay = l00r * x.y + l00i * x.x + sgn * (l01r * y.y + l01i * y.x);
                      bxr = sgn * (l10r * x.x - l10i * x.y) + l11r * y.x - l11i * y.y;
                      byi = sgn * (l10r * x.y + l10i * x.x) + l11r * y.y + l11i * y.x;
                    }
                    float2 nx, ny;
                    nx.x = g00r * x.x - g00i * x.y + sgn * (g01r * y.x - g01i * y.y) + ax;
                    nx.y = g00r * x.y + g00i * x.x + sgn * (g01r * y.y + g01i * y.x) + ay;
                    ny.x = sgn * (g10r * x.x - g10i * x.y) + g11r * y.x - g11i * y.y + bxr;
                    ny.y = sgn * (g10r * x.y + g10i * x.x) + g11r * y.y + g11i * y.x + byi;
                    bx[j] = nx;
                    by[jp] = ny;
                  }
                };
                if (comp)
                  run(std::true_type{});
                else
                  run(std::false_type{});
              });
          __syncthreads();
        }
        low_stage(wp + 2 * 84);
        high_stage(wp + 3 * 84);
      }
    }

    // ----------------------------------------------------------- epilogue
    for (int rho = 0; rho < R; ++rho) {
      const long long r = row0 + rho;
      if (P.diag_mode != DIAG_NONE) {
        const unsigned rs = P.row_strings[r];
        const int rn = P.row_norb;
        // m[l] = sum_i cross[i][l] g_i(r); sM[0..norb) = weights, sM[MAXN] = row part
        if (tid < norb) {
          double m = 0.0;
          for (int i = 0; i < rn; ++i) {
            const double gi = P.zrep ? ((rs >> i) & 1u ? -1.0 : 1.0) : (double)((rs >> i) & 1u);
            m += P.cross[i][tid] * gi;
          }
          sM[tid] = m;
        }
        if (tid == 32) {
          double f = 0.0;
          for (int i = 0; i < rn; ++i) {
            const double gi = P.zrep ? ((rs >> i) & 1u ? -1.0 : 1.0) : (double)((rs >> i) & 1u);
            if (gi == 0.0) continue;
            for (int i2 = i; i2 < rn; ++i2) {
              const double gj = P.zrep ? ((rs >> i2) & 1u ? -1.0 : 1.0) : (double)((rs >> i2) & 1u);
              f += P.rsame[i][i2] * gi * gj;
            }
          }
          sM[FFGB_MAXN] = f;
        }
        __syncthreads();
        if (tid == 0) {
          double f = sM[FFGB_MAXN];
          if (P.zrep)
            for (int l = 0; l < norb; ++l) f += sM[l];
          sM[FFGB_MAXN + 1] = f;
        }
        __syncthreads();
        const double wsc = P.zrep ? -2.0 : 1.0;
        const double rc = sM[FFGB_MAXN + 1];
        for (int e = tid; e < nent; e += nth) {
          const int c = e >> cb;
          unsigned x = (unsigned)(e & cmask);
          double f = (c == 0) ? rc : 0.0;
          while (x) {
            const int b = __ffs(x) - 1;
            x &= x - 1;
            const int orb = c * cb + b;
            if (orb < norb) f += wsc * sM[orb];
          }
          if (P.diag_mode == DIAG_PHASE) {
            C ph = phase_of(f, (C*)nullptr);
            if (P.has_dphase) {
              unsigned y = (unsigned)(e & cmask);
              while (y) {
                const int b = __ffs(y) - 1;
                y &= y - 1;
                const int orb = c * cb + b;
                if (orb < norb) {
                  C d;
                  d.x = P.dphase[orb][0];
                  d.y = P.dphase[orb][1];
                  ph = cmul(ph, d);
                }
              }
            }
            sXP[e] = ph;
          } else {
            sXC[e] = (T)f;
          }
        }
        __syncthreads();
      }
      const C* vr = srow + (long long)rho * dim;
      const bool need_s = P.has_dphase || P.diag_mode != DIAG_NONE;
      const unsigned* __restrict__ cstr = P.col_strings;
      constexpr int U = 4;  // elements per thread per step: their global loads overlap
      for (int j0 = tid; j0 < dim; j0 += U * nth) {
        unsigned sv[U];
        C cp[U];
        T cz[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int j = j0 + u * nth;
          sv[u] = 0;
          cz[u] = (T)0;
          cp[u] = cmake<C>(1.0, 0.0);
          if (j < dim) {
            if (need_s) sv[u] = __ldg(cstr + j);
            if (P.diag_mode == DIAG_PHASE && colP) cp[u] = colP[j];
            if (P.diag_mode == DIAG_COEF && colZ) cz[u] = colZ[j];
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int j = j0 + u * nth;
          if (j >= dim) break;
          C v = vr[j];
          const unsigned s = sv[u];
          if (sep_dphase) {
            for (int c = 0; c < dch; ++c) v = cmul(v, sDT[(c << 4) + ((s >> (c * 4)) & 15u)]);
          }
          T z = (T)1;
          if (P.diag_mode == DIAG_PHASE) {
            C f = cp[u];
            for (int c = 0; c < nch; ++c) f = cmul(f, sXP[(c << cb) + ((s >> (c * cb)) & cmask)]);
            v = cmul(v, f);
          } else if (P.diag_mode == DIAG_COEF) {
            z = cz[u];
            for (int c = 0; c < nch; ++c) z += sXC[(c << cb) + ((s >> (c * cb)) & cmask)];
            if (P.out_op != OUT_EXPECT) {
              v.x *= z;
              v.y *= z;
            }
          }
          if (P.out_op == OUT_EXPECT) {
            const T w = (v.x * v.x + v.y * v.y) * z;
            if constexpr (sizeof(T) == 4) {
              const float y = (float)w - comp_f;
              const float t = acc_f + y;
              comp_f = (t - acc_f) - y;
              acc_f = t;
            } else {
              acc_d += (double)w;
            }
          } else if (P.out_op != OUT_NONE) {
            const long long o = (P.layout == LAYOUT_SAME) ? r * (long long)dim + j : (long long)j * P.n_rows + r;
            if (P.out_op == OUT_STORE) {
              out[o] = v;
            } else {
              C a = out[o];
              a.x += P.alpha_re * v.x - P.alpha_im * v.y;
              a.y += P.alpha_re * v.y + P.alpha_im * v.x;
              out[o] = a;
            }
          }
        }
      }
      if (P.diag_mode != DIAG_NONE) __syncthreads();
    }
    if constexpr (sizeof(T) == 4) {
      // fold the FP32 partial into FP64 once per chunk
      acc_d += (double)acc_f - (double)comp_f;
      acc_f = 0.f;
      comp_f = 0.f;
    }
    __syncthreads();  // the next chunk overwrites the staged rows
  }

  if (P.out_op == OUT_EXPECT) {
    double a = acc_d;
    for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
    if ((tid & 31) == 0) sRed[tid >> 5] = a;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int w = 0; w < (nth >> 5); ++w) s += sRed[w];
      P.partials[blockIdx.x] = s;
    }
  }
}


// One adjacent rotation on one spin sector directly in global memory (the
// counterpart of the reference's per-Givens row-pair sweep).  spin 0: the
// sector indexes rows (stride dim_other), spin 1: columns.
template <typename T>
__global__ void givens_sector_kernel(typename CT<T>::type* __restrict__ vec, int norb, int nocc,
                                     long long dim_other, int spin, int l, T c, T sr, T si) {
  using C = typename CT<T>::type;
  __shared__ int sB[FFGB_BST * FFGB_BST];
  for (int idx = threadIdx.x; idx < FFGB_BST * FFGB_BST; idx += blockDim.x) {
    int a = idx / FFGB_BST, b = idx % FFGB_BST;
    long long r = 0;
    if (b <= a) {
      r = 1;
      for (int i = 1; i <= b; ++i) r = r * (a - b + i) / i;
    }
    sB[idx] = (int)r;
  }
  __syncthreads();
  if (nocc < 1 || nocc > norb - 1) return;
  const long long npairs = bn(sB, norb - 2, nocc - 1);
  const long long total = npairs * dim_other;
  const int dim = bn(sB, norb, nocc);
  const unsigned lowmask = (1u << l) - 1u;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    long long t, o;
    if (spin == 0) {
      t = idx / dim_other;
      o = idx - t * dim_other;
    } else {
      o = idx / npairs;
      t = idx - o * npairs;
    }
    const unsigned p = unrank_colex((int)t, norb - 2, nocc - 1, sB);
    const unsigned x = (p & lowmask) | (1u << l) | ((p >> l) << (l + 2));
    const int rx = rank_colex(x, sB);
    const int ry = rx + bn(sB, l, __popc(p & lowmask));
    const long long ax = spin == 0 ? (long long)rx * dim_other + o : o * dim + rx;
    const long long ay = spin == 0 ? (long long)ry * dim_other + o : o * dim + ry;
    C a = vec[ax], b = vec[ay], na, nb;
    na.x = c * a.x + sr * b.x - si * b.y;
    na.y = c * a.y + sr * b.y + si * b.x;
    nb.x = c * b.x - sr * a.x - si * a.y;
    nb.y = c * b.y - sr * a.y + si * a.x;
    vec[ax] = na;
    vec[ay] = nb;
  }
}

// Multiply every amplitude whose sector string has orbital `orb` occupied.
template <typename T>
__global__ void phase_shift_kernel(typename CT<T>::type* __restrict__ vec, const unsigned* __restrict__ strings,
                                   long long dim_a, long long dim_b, int spin, int orb, T pr, T pi) {
  using C = typename CT<T>::type;
  const long long total = dim_a * dim_b;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long a = idx / dim_b, b = idx - a * dim_b;
    const unsigned s = strings[spin == 0 ? a : b];
    if ((s >> orb) & 1u) {
      C v = vec[idx], o;
      o.x = pr * v.x - pi * v.y;
      o.y = pr * v.y + pi * v.x;
      vec[idx] = o;
    }
  }
}

// out = a+_{p spin} a_{q spin} in: each string with q occupied and p empty (or
// p == q) moves to the string with q emptied and p filled, with the sign of the
// occupied orbitals below q (annihilation) and below p after it (creation).
// The map is injective for fixed (p, q), so every target is written once;
// targets without a source keep the zeros the caller wrote.
template <typename T>
__global__ void excitation_kernel(const typename CT<T>::type* __restrict__ in, typename CT<T>::type* __restrict__ out,
                                  const unsigned* __restrict__ strings, long long dim_a, long long dim_b, int spin,
                                  int p, int q) {
  using C = typename CT<T>::type;
  __shared__ int sB[FFGB_BST * FFGB_BST];
  for (int idx = threadIdx.x; idx < FFGB_BST * FFGB_BST; idx += blockDim.x) {
    const int a = idx / FFGB_BST, b = idx % FFGB_BST;
    long long r = 0;
    if (b <= a) {
      r = 1;
      for (int i = 1; i <= b; ++i) r = r * (a - b + i) / i;
    }
    sB[idx] = (int)r;
  }
  __syncthreads();
  const long long total = dim_a * dim_b;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long a = idx / dim_b, b = idx - a * dim_b;
    const unsigned s = strings[spin == 0 ? a : b];
    if (!((s >> q) & 1u)) continue;
    const unsigned mid = s & ~(1u << q);
    if (p != q && ((mid >> p) & 1u)) continue;
    const unsigned t = mid | (1u << p);
    const int parity = (__popc(s & ((1u << q) - 1u)) + __popc(mid & ((1u << p) - 1u))) & 1;
    const long long r = rank_colex(t, sB);
    const long long dst = spin == 0 ? r * dim_b + b : a * dim_b + r;
    C v = in[idx];
    if (parity) {
      v.x = -v.x;
      v.y = -v.y;
    }
    out[dst] = v;
  }
}

// F_C(j) of the rotated sector: phase exp(i F) (mode 1) or coefficient F (mode 2)
// Same-sector coefficients of a diagonal operator, passed by value as a
// kernel parameter (no device copy, nothing read from host memory).
struct SameTable {
  double v[FFGB_MAXN * FFGB_MAXN];
};

template <typename T>
__global__ void col_table_kernel(const unsigned* __restrict__ strings, int dim, int norb, int zrep,
                                 int mode, const __grid_constant__ SameTable same, void* out) {
  using C = typename CT<T>::type;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= dim) return;
  const unsigned s = strings[j];
  double f = 0.0;
  for (int i = 0; i < norb; ++i) {
    const double gi = zrep ? ((s >> i) & 1u ? -1.0 : 1.0) : (double)((s >> i) & 1u);
    if (gi == 0.0) continue;
    for (int i2 = i; i2 < norb; ++i2) {
      const double gj = zrep ? ((s >> i2) & 1u ? -1.0 : 1.0) : (double)((s >> i2) & 1u);
      f += same.v[i * FFGB_MAXN + i2] * gi * gj;
    }
  }
  if (mode == DIAG_PHASE)
    ((C*)out)[j] = phase_of(f, (C*)nullptr);
  else
    ((T*)out)[j] = (T)f;
}

// deterministic sum of n doubles into out[slot]
static __global__ void reduce_partials_kernel(const double* __restrict__ in, long long n, double* out, int slot) {
  __shared__ double sh[256];
  double a = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) a += in[i];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[slot] = sh[0];
}

// partial sums of conj(x) y per CTA
template <typename T>
__global__ void vdot_kernel(const typename CT<T>::type* __restrict__ x,
                            const typename CT<T>::type* __restrict__ y, long long n,
                            double* __restrict__ partials) {
  __shared__ double sr[32], si[32];
  double ar = 0.0, ai = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double xr = x[i].x, xi = x[i].y, yr = y[i].x, yi = y[i].y;
    ar += xr * yr + xi * yi;
    ai += xr * yi - xi * yr;
  }
  for (int off = 16; off > 0; off >>= 1) {
    ar += __shfl_down_sync(0xffffffffu, ar, off);
    ai += __shfl_down_sync(0xffffffffu, ai, off);
  }
  if ((threadIdx.x & 31) == 0) {
    sr[threadIdx.x >> 5] = ar;
    si[threadIdx.x >> 5] = ai;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += sr[w];
      b += si[w];
    }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
}

template <typename T>
__global__ void scale_copy_kernel(const typename CT<T>::type* __restrict__ x,
                                  typename CT<T>::type* __restrict__ y, long long n, T ar, T ai) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    typename CT<T>::type v = x[i], o;
    o.x = ar * v.x - ai * v.y;
    o.y = ar * v.y + ai * v.x;
    y[i] = o;
  }
}

template <typename T>
__global__ void one_hot_kernel(typename CT<T>::type* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    typename CT<T>::type v;
    v.x = (i == 0) ? (T)1 : (T)0;
    v.y = (T)0;
    y[i] = v;
  }
}

}  // namespace ffgb
