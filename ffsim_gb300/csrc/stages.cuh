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
  // states side by side along the columns: column c is string c mod
  // col_period of its state (0: one state); padded columns (string index
  // >= col_valid) hold zero amplitudes and read the last string's entries
  long long col_period, col_valid;
  float X[FFGB_MAXN][FFGB_MAXN];
  float Xsum[FFGB_MAXN];  // sum_i X[i][l]
  int zrep;
};

// One launch of a window stage: the groups of one electron-count class K
// (KIND 0: plain members; KIND 1: K = B/2, complement-packed within the
// group), or pairs of groups of classes K and B - K (KIND 2, complement-packed
// across the two groups).
struct WinJob {
  const float2* in;
  float2* out;
  long long ld;     // row stride (elements)
  long long ncols;  // columns processed
  int tiles;        // column tiles per group
  int norb, lo;     // orbitals; first orbital of the window
  const int* gbase_a;  // base row of every group of class K (device table)
  const int* gbase_b;  // and of the paired class B - K (packed launches)
  int off_a[72], off_b[72];    // member row offsets from the base row (windows not starting at orbital 0)
  long long eoff_a[72], eoff_b[72];  // the same times ld: element offsets, so an address is one add
  float gp[84], gl[84];        // window network coefficients (see win_coef)
  unsigned gt[84];
  unsigned salt;
  long long col_period;  // > 0: the dithering of column c is that of column c mod col_period
  StageExpect ex;        // partials of this launch start at ex.partials
  int n_groups;          // groups (or group pairs) of this launch
};

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Registers: the members of one thread are 2 * C(B, K) floats (twice that for
// KIND 2); addressing, coefficients and scheduling slack take about
// 30 + 0.55 * data more (measured with -Xptxas -v), the fused expectation ~16.
__host__ __device__ constexpr int win_min_blocks(int b, int k, int kind, int epi) {
  const int data = 2 * win_members(b, k) * (kind == 2 ? 2 : 1);
  const int need = 30 + (155 * data) / 100 + (epi == 2 ? 16 : 0);
  return need <= 64 ? 8 : need <= 80 ? 6 : need <= 96 ? 5 : need <= 128 ? 4 : need <= 168 ? 3 : 2;
}

// Per-thread part of the fused expectation: weights of the window orbitals
// (sum_l X[lo + t][l] g_l(col)) and the constant part of z for one group.
struct ZCtx {
  float w[8];
  float base, scale;
};

// xw[t][l] = X[lo + t][l] (rows of FFGB_MAXN), xs[l] = sum_i X[i][l], and
// ya[l], yb[l] = sum over the group's electrons outside the window of X[i][l]:
// per-CTA tables in shared memory.
template <int B>
__device__ __forceinline__ void zctx_make(const float* xw, const float* xs, const float* ya, const float* yb, int norb,
                                          int zrep, unsigned cstr, ZCtx& za, ZCtx& zb, float zc) {
  float sa = 0.f, sb = 0.f, wall = 0.f;
#pragma unroll
  for (int t = 0; t < B; ++t) za.w[t] = 0.f;
  for (int l = 0; l < norb; ++l) {
    const float gcol = zrep ? (((cstr >> l) & 1u) ? -1.f : 1.f) : (float)((cstr >> l) & 1u);
#pragma unroll
    for (int t = 0; t < B; ++t) za.w[t] += xw[t * FFGB_MAXN + l] * gcol;
    sa += ya[l] * gcol;
    sb += yb[l] * gcol;
    wall += xs[l] * gcol;
  }
#pragma unroll
  for (int t = 0; t < B; ++t) zb.w[t] = za.w[t];
  if (zrep) {
    za.base = zc + wall - 2.f * sa;
    zb.base = zc + wall - 2.f * sb;
    za.scale = zb.scale = -2.f;
  } else {
    za.base = zc + sa;
    zb.base = zc + sb;
    za.scale = zb.scale = 1.f;
  }
}

template <int B>
__device__ __forceinline__ float zpat(const ZCtx& z, unsigned pat, float zrow) {
  float ws = 0.f;
#pragma unroll
  for (int t = 0; t < B; ++t)
    if ((pat >> t) & 1u) ws += z.w[t];
  return zrow + z.base + z.scale * ws;
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

// Kahan step in FP32.
__device__ __forceinline__ void kahan_add(float& acc, float& cmp, float v) {
  const float y = v - cmp;
  const float t = acc + y;
  cmp = (t - acc) - y;
  acc = t;
}

// Epilogues of a window stage: store, or the fused expectation (nothing stored).
enum { EPI_STORE = 0, EPI_EXPECT = 2 };

template <int B, int K, int KIND, bool LOW, int EPI>
__global__ void __launch_bounds__(STAGE_THREADS, win_min_blocks(B, K, KIND, EPI))
    win_class_kernel(const __grid_constant__ WinJob P) {
  constexpr int MODE = 2;
  constexpr bool EXPECT = EPI == EPI_EXPECT;
  const int g = blockIdx.x / P.tiles, tile = blockIdx.x - g * P.tiles;
  const long long col = (long long)tile * STAGE_THREADS + threadIdx.x;
  const bool active = col < P.ncols;
  if (!EXPECT && !active) return;
  const long long ra = P.gbase_a[g];
  const long long rb = P.gbase_b ? (long long)P.gbase_b[g] : ra;
  unsigned rng = dither_seed((unsigned long long)(P.col_period ? col % P.col_period : col), P.salt);
  const long long ld = P.ld;
  // string index of this column (states side by side along the columns)
  const long long cidx = !EXPECT || !P.ex.col_period ? col : min(col % P.ex.col_period, P.ex.col_valid - 1);
  // member j of group A (class K) / group B (class B - K): row offset from the group's base
#define ROW_A(j) (LOW ? (long long)(j) : (long long)P.off_a[(j)])
#define ROW_B(j) (LOW ? (long long)(j) : (long long)P.off_b[(j)])
  // element offsets of member j for the leading dimension `l`
#define EL_A(j, l) (LOW ? (long long)(j) * (l) : P.eoff_a[(j)])
#define EL_B(j, l) (LOW ? (long long)(j) * (l) : P.eoff_b[(j)])
  double part = 0.0;
  // fused expectation: the operator's weights for this CTA's group(s), once per CTA
  constexpr int XS = EXPECT ? FFGB_MAXN : 1;
  __shared__ float sxw[EXPECT ? B * FFGB_MAXN : 1], sxs[XS], sya[XS], syb[XS];
  if constexpr (EXPECT) {
    const unsigned wmask = ((1u << B) - 1u) << P.lo;
    const unsigned out_a = P.ex.row_str[ra + ROW_A(0)] & ~wmask;
    const unsigned out_b = KIND == 2 ? (P.ex.row_str[rb + ROW_B(0)] & ~wmask) : out_a;
    const int n = P.norb;
    for (int e = threadIdx.x; e < (B + 3) * n; e += STAGE_THREADS) {
      const int row = e / n, l = e - row * n;
      if (row < B) {
        sxw[row * FFGB_MAXN + l] = P.ex.X[P.lo + row][l];
      } else if (row == B) {
        sxs[l] = P.ex.Xsum[l];
      } else {
        const unsigned o = row == B + 1 ? out_a : out_b;
        float y = 0.f;
        for (int i = 0; i < n; ++i)
          if ((o >> i) & 1u) y += P.ex.X[i][l];
        (row == B + 1 ? sya : syb)[l] = y;
      }
    }
    __syncthreads();
  }
  if (active) {
    const float2* sa = P.in + ra * ld + col;
    const float2* sb = P.in + rb * ld + col;
    if constexpr (KIND == 0) {
      constexpr int M = WinNet<B, K>::M;
      float2 v[M];
#pragma unroll
      for (int j = 0; j < M; ++j) v[j] = sa[EL_A(j, ld)];
      WinNet<B, K>::template apply<MODE>(v, P.gp, P.gl, P.gt, rng);
      if constexpr (!EXPECT) {
        // fresh copies: keeps the compiler from holding every member's offset
        // live from the loads to the stores
        float2* da = P.out + ra * ld + col;
        long long ls = ld;
        asm volatile("" : "+l"(da), "+l"(ls));
#pragma unroll
        for (int j = 0; j < M; ++j) da[EL_A(j, ls)] = v[j];
      } else {
        const StageExpect& E = P.ex;
        ZCtx za, zb;
        zctx_make<B>(sxw, sxs, sya, sya, P.norb, E.zrep, E.col_str[cidx], za, zb, E.zcol[cidx]);
        float acc = 0.f, cmp = 0.f;
        // member patterns in colex order = ascending integers with K bits set,
        // stepped with the next-same-popcount recurrence (folds to constants)
        unsigned pat = (1u << K) - 1u;
#pragma unroll
        for (int j = 0; j < M; ++j) {
          const float z = zpat<B>(za, pat, __ldg(E.zrow + ra + ROW_A(j)));
          kahan_add(acc, cmp, z * (v[j].x * v[j].x + v[j].y * v[j].y));
          if (j + 1 < M) {
            const unsigned low = pat & (0u - pat), r = pat + low;
            pat = (((r ^ pat) >> 2) / low) | r;
          }
        }
        part = (double)acc - (double)cmp;
      }
    } else {
      using PK = WinPack<B, K>;
      constexpr int NP = PK::NP;
      constexpr bool PAIR = KIND == 2;
      const float2* s1 = PAIR ? sb : sa;
      const long long r1 = PAIR ? rb : ra;
      float2 R[NP], I[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const float2 a = sa[EL_A(PK::lane0(q), ld)];
        const float2 b = s1[PAIR ? EL_B(PK::lane1(q), ld) : EL_A(PK::lane1(q), ld)];
        R[q] = make_float2(a.x, b.x);
        I[q] = make_float2(a.y, b.y);
      }
      PK::template apply<MODE>(R, I, P.gp, P.gl, P.gt, rng);
      if constexpr (!EXPECT) {
        float2* da = P.out + ra * ld + col;
        float2* db = P.out + r1 * ld + col;
        long long ls = ld;
        asm volatile("" : "+l"(da), "+l"(db), "+l"(ls));
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          const long long o0 = EL_A(PK::lane0(q), ls), o1 = PAIR ? EL_B(PK::lane1(q), ls) : EL_A(PK::lane1(q), ls);
          da[o0] = make_float2(R[q].x, I[q].x);
          db[o1] = make_float2(R[q].y, I[q].y);
        }
      } else {
        const StageExpect& E = P.ex;
        ZCtx za, zb;
        zctx_make<B>(sxw, sxs, sya, syb, P.norb, E.zrep, E.col_str[cidx], za, zb, E.zcol[cidx]);
        float acc = 0.f, cmp = 0.f;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          const float z0 = zpat<B>(za, PK::pat0(q), __ldg(E.zrow + ra + ROW_A(PK::lane0(q))));
          const float z1 = zpat<B>(PAIR ? zb : za, PK::pat1(q),
                                   __ldg(E.zrow + r1 + (PAIR ? ROW_B(PK::lane1(q)) : ROW_A(PK::lane1(q)))));
          const float2 m2 = __ffma2_rn(R[q], R[q], __fmul2_rn(I[q], I[q]));
          kahan_add(acc, cmp, z0 * m2.x);
          kahan_add(acc, cmp, z1 * m2.y);
        }
        part = (double)acc - (double)cmp;
      }
    }
  }
#undef ROW_A
#undef ROW_B
#undef EL_A
#undef EL_B
  if constexpr (EXPECT) {
    __shared__ double sh[STAGE_THREADS / 32];
    const double s = block_sum_128(part, sh);
    if (threadIdx.x == 0) P.ex.partials[blockIdx.x] = s;
  }
}

// Cross-half rotations (lo + i, lo + hh + i) of all sites in one pass.  A
// group is the set of strings that agree everywhere except in which orbital of
// each "active" pair (exactly one of the two occupied) is occupied: 2^M members
// for M active sites, held in registers for M <= CS_MAX_M.  Table entry per group: a header with the active sites
// (4 bits each, ascending), then per member its row | (sign bits << 24); bit
// 24 + t is the parity of the occupied orbitals strictly between the two
// orbitals of active site t, read on the member whose lower orbital is
// occupied.  Pairs with both or neither orbital occupied are left alone: the
// 2x2 blocks of the plan have determinant 1.
constexpr int CS_MAX_GPC = 8;     // groups per CTA of the cross-half stage (at most)
constexpr int CS_MAX_SITES = 12;  // cross-half sites of one stage (at most)
constexpr int CS_MAX_M = 6;       // active sites of a group kept in registers

struct CsStageParams {
  float2* x;
  long long ld, ncols;
  const int* tab;  // this class's groups, (1 + 2^M) ints each
  int n_groups;
  int tiles;
  int gpc;  // groups per CTA (one column tile each): an even number <= CS_MAX_GPC, at most half that for M >= 5
  float gp[3 * CS_MAX_SITES], gl[3 * CS_MAX_SITES];  // per site (c, Re t, Im t), see win_coef
  unsigned gt[3 * CS_MAX_SITES];
  unsigned salt;
  long long col_period;  // > 0: the dithering of column c is that of column c mod col_period
};

// One group's cross-half rotations on registers; e[j] = row | sign bits.
template <int M, int MODE>
__device__ __forceinline__ void cs_rotate(float2 (&v)[1 << M], const int* e, int sites,
                                          const float* __restrict__ gp, const float* __restrict__ gl,
                                          const unsigned* __restrict__ gt, unsigned rng) {
  constexpr int NM = 1 << M;
#pragma unroll
  for (int t = 0; t < M; ++t) {
    const int site = (sites >> (4 * t)) & 15;
    float c, sr, si, cl, srl, sil;
    win_coef<MODE>(gp, gl, gt, site, rng, c, sr, si, cl, srl, sil);
#pragma unroll
    for (int j = 0; j < NM; ++j) {
      if (j & (1 << t)) continue;
      const float sg = ((e[j] >> (24 + t)) & 1) ? -1.f : 1.f;
      rot_pair<MODE == 1>(v[j], v[j | (1 << t)], c, sg * sr, sg * si, cl, sg * srl, sg * sil);
    }
  }
}

// Groups with M active sites.  For M <= 4 each thread takes two groups at a
// time so that both groups' loads are in flight together; larger groups (up to
// 64 members) go one at a time.  The member tables stay in shared memory.
template <int M, int MODE>
__global__ void __launch_bounds__(STAGE_THREADS, M >= 5 ? 3 : (M >= 4 ? 4 : 6))
    cs_stage_kernel(const __grid_constant__ CsStageParams P) {
  constexpr int NM = 1 << M;
  constexpr int STRIDE = 1 + NM;
  constexpr bool TWO = M <= 4;
  constexpr int GPC = TWO ? CS_MAX_GPC : CS_MAX_GPC / 2;
  const int chunk = blockIdx.x / P.tiles, tile = blockIdx.x - chunk * P.tiles;
  const long long col = (long long)tile * STAGE_THREADS + threadIdx.x;
  const int g0 = chunk * P.gpc, g1 = min(g0 + P.gpc, P.n_groups);
  // this CTA's group tables, staged once in shared memory
  __shared__ int sent[GPC * STRIDE];
  const int n_ent = (g1 - g0) * STRIDE;
  const int* src = P.tab + (long long)g0 * STRIDE;
  for (int i = threadIdx.x; i < n_ent; i += STAGE_THREADS) sent[i] = src[i];
  __syncthreads();
  if (col >= P.ncols) return;
  const unsigned rng = dither_seed((unsigned long long)(P.col_period ? col % P.col_period : col), P.salt);
  float2* xc = P.x + col;
  const long long ld = P.ld;
  for (int g = g0; g < g1; g += TWO ? 2 : 1) {
    const bool two = TWO && g + 1 < g1;
    const int* ea = sent + (g - g0) * STRIDE;
    const int* eb = two ? ea + STRIDE : ea;
    float2 v0[NM], v1[TWO ? NM : 1];
#pragma unroll
    for (int j = 0; j < NM; ++j) v0[j] = xc[(long long)(ea[1 + j] & 0xffffff) * ld];
    if constexpr (TWO) {
      if (two) {
#pragma unroll
        for (int j = 0; j < NM; ++j) v1[j] = xc[(long long)(eb[1 + j] & 0xffffff) * ld];
      }
    }
    cs_rotate<M, MODE>(v0, ea + 1, ea[0], P.gp, P.gl, P.gt, rng);
    // re-read the rows from shared memory for the stores instead of keeping
    // 2^M addresses live across the rotations
    asm volatile("" ::: "memory");
#pragma unroll
    for (int j = 0; j < NM; ++j) xc[(long long)(ea[1 + j] & 0xffffff) * ld] = v0[j];
    if constexpr (TWO) {
      if (two) {
        cs_rotate<M, MODE>(v1, eb + 1, eb[0], P.gp, P.gl, P.gt, rng);
#pragma unroll
        for (int j = 0; j < NM; ++j) xc[(long long)(eb[1 + j] & 0xffffff) * ld] = v1[j];
      }
    }
  }
}

// Groups with M = 5 or 6 active sites on two lanes per column: lane 2c holds
// the members with the last active site's bit clear, lane 2c + 1 the others,
// so a thread keeps 2^(M-1) amplitudes (four CTAs per SM instead of three).
// The sites below the last act within a lane; the last one pairs member j of
// the even lane with member j of the odd lane through a shuffle.  Both lanes
// of a column draw the same dithered coefficients, in the same order as
// cs_rotate, and the arithmetic of every pair is rot_pair's, so the result
// equals cs_stage_kernel's.  A CTA covers 64 columns (P.tiles counts 64-column
// tiles); columns beyond ncols run on zeros and store nothing.
template <int M, int MODE>
__global__ void __launch_bounds__(STAGE_THREADS, 4) cs_pair_kernel(const __grid_constant__ CsStageParams P) {
  static_assert(M >= 2 && MODE != 1, "plain or dithered coefficients, at least two sites");
  constexpr int NM = 1 << M, NH = NM / 2, STRIDE = 1 + NM, TL = M - 1;
  constexpr int GPC = CS_MAX_GPC / 2;
  const int chunk = blockIdx.x / P.tiles, tile = blockIdx.x - chunk * P.tiles;
  const int half = threadIdx.x & 1;
  const long long col = (long long)tile * (STAGE_THREADS / 2) + (threadIdx.x >> 1);
  const int g0 = chunk * P.gpc, g1 = min(g0 + P.gpc, P.n_groups);
  __shared__ int sent[GPC * STRIDE];
  const int n_ent = (g1 - g0) * STRIDE;
  const int* src = P.tab + (long long)g0 * STRIDE;
  for (int i = threadIdx.x; i < n_ent; i += STAGE_THREADS) sent[i] = src[i];
  __syncthreads();
  const bool active = col < P.ncols;
  const unsigned rng = dither_seed((unsigned long long)(P.col_period ? col % P.col_period : col), P.salt);
  float2* xc = P.x + (active ? col : 0);
  const long long ld = P.ld;
  for (int g = g0; g < g1; ++g) {
    const int* e = sent + (g - g0) * STRIDE;
    const int sites = e[0];
    const int* em = e + 1;
    float2 v[NH];
#pragma unroll
    for (int j = 0; j < NH; ++j)
      v[j] = active ? xc[(long long)(em[half * NH + j] & 0xffffff) * ld] : make_float2(0.f, 0.f);
    unsigned r = rng;
#pragma unroll
    for (int t = 0; t < TL; ++t) {
      const int site = (sites >> (4 * t)) & 15;
      float c, sr, si, cl, srl, sil;
      win_coef<MODE>(P.gp, P.gl, P.gt, site, r, c, sr, si, cl, srl, sil);
#pragma unroll
      for (int j = 0; j < NH; ++j) {
        if (j & (1 << t)) continue;
        const float sg = ((em[half * NH + j] >> (24 + t)) & 1) ? -1.f : 1.f;
        rot_pair<false>(v[j], v[j | (1 << t)], c, sg * sr, sg * si, 0.f, 0.f, 0.f);
      }
    }
    {
      const int site = (sites >> (4 * TL)) & 15;
      float c, sr, si, cl, srl, sil;
      win_coef<MODE>(P.gp, P.gl, P.gt, site, r, c, sr, si, cl, srl, sil);
#pragma unroll
      for (int j = 0; j < NH; ++j) {
        // the sign is read on the member whose lower orbital is occupied: the even lane's
        const float sg = ((em[j] >> (24 + TL)) & 1) ? -1.f : 1.f;
        const float2 o = make_float2(__shfl_xor_sync(0xffffffffu, v[j].x, 1), __shfl_xor_sync(0xffffffffu, v[j].y, 1));
        if (half == 0)
          rot_half_x(v[j], o, c, sg * sr, sg * si);
        else
          rot_half_y(v[j], o, c, sg * sr, sg * si);
      }
    }
    if (active) {
#pragma unroll
      for (int j = 0; j < NH; ++j) xc[(long long)(em[half * NH + j] & 0xffffff) * ld] = v[j];
    }
  }
}

// out[c][r] = in[r][c] * row_ph[r] * col_ph[c] (phase tables optional), row
// strides ld_in / ld_out.  A CTA moves a 64-row x 32-column tile through
// shared memory (padded rows: no bank conflicts); each thread has eight loads
// in flight.  blockIdx.z indexes states side by side along the columns of
// both arrays: state z starts at column z * in_step of `in` and z * out_step
// of `out`.
template <typename C>
__global__ void __launch_bounds__(256) transpose_kernel(const C* __restrict__ in, C* __restrict__ out,
                                                        long long rows, long long cols, long long ld_in,
                                                        long long ld_out, long long in_step, long long out_step,
                                                        const C* __restrict__ row_ph,
                                                        const C* __restrict__ col_ph) {
  __shared__ C tile[64][33];
  in += (long long)blockIdx.z * in_step;
  out += (long long)blockIdx.z * out_step;
  const long long c0 = (long long)blockIdx.x * 32, r0 = (long long)blockIdx.y * 64;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
  for (int j = ty; j < 64; j += 8) {
    const long long r = r0 + j, c = c0 + tx;
    if (r < rows && c < cols) {
      C v = in[r * ld_in + c];
      if (row_ph) v = cmul(v, row_ph[r]);
      if (col_ph) v = cmul(v, col_ph[c]);
      tile[j][tx] = v;
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = ty; j < 32; j += 8) {
    const long long c = c0 + j;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long r = r0 + tx + 32 * h;
      if (c < cols && r < rows) out[c * ld_out + r] = tile[tx + 32 * h][j];
    }
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

// y += ph[row] * x over rows of length ld (ph optional: y += x)
template <typename C>
__global__ void row_axpy_kernel(const C* __restrict__ x, C* __restrict__ y, long long rows, long long ld,
                                const C* __restrict__ ph) {
  const long long n = rows * ld;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const C v = ph ? cmul(x[i], ph[i / ld]) : x[i];
    C o = y[i];
    o.x += v.x;
    o.y += v.y;
    y[i] = o;
  }
}

// States side by side along the columns ("stacked"): state b of a block of
// contiguous states x[b][r][c] (rows x cols each) is columns
// [b * pad, b * pad + cols) of y[r][...] (row stride n_states * pad).
// dir 0: y <- x (padding columns untouched); dir 1: x <- y, or x += y with
// accumulate.
template <typename C>
__global__ void stack_kernel(C* __restrict__ x, C* __restrict__ y, long long n_states, long long rows,
                             long long cols, long long pad, int dir, int accumulate) {
  const long long per = rows * cols, n = n_states * per, ld = n_states * pad;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / per, rem = i - b * per, r = rem / cols, c = rem - r * cols;
    C* yy = y + r * ld + b * pad + c;
    if (dir == 0) {
      *yy = x[i];
    } else if (accumulate) {
      C o = x[i];
      const C v = *yy;
      o.x += v.x;
      o.y += v.y;
      x[i] = o;
    } else {
      x[i] = *yy;
    }
  }
}

// Per-state sums of the fused expectation's per-CTA partials for stacked
// states: partial p of a stage belongs to column tile p mod tiles, and tile
// t to state t / tiles_per_state.  Block b sums its state's partials in a
// fixed order into out[b].
static __global__ void __launch_bounds__(256) state_partials_kernel(const double* __restrict__ partials, long long n,
                                                             long long tiles, long long tiles_per_state,
                                                             double* __restrict__ out) {
  __shared__ double sh[256];
  const long long b = blockIdx.x;
  double a = 0.0;
  for (long long p = threadIdx.x; p < n; p += blockDim.x)
    if ((p % tiles) / tiles_per_state == b) a += partials[p];
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[b] = sh[0];
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
