// Diagonal operators streamed row by row: no shared-memory copy of a row, so
// every sector size fits.  For a state whose rows are strings of one sector
// and whose columns are strings of the other,
//   f(r, c) = F_R(r) + F_C(c) + sum_{i,l} X[i][l] g_i(r) g_l(c),
// g = n (number representation) or 1 - 2n (Z representation).  Per row the
// FP64 row term and the weights m_l(r) = sum_i X[i][l] g_i(r) are formed once
// and tabulated over the halves of the column string (below); per element the
// column term comes from a table (exp(i F_C) for phases, F_C for coefficients).
#pragma once

#include "kernels.cuh"

namespace ffgb {

constexpr int DIAG_THREADS = 256;
constexpr int DIAG_ROWS_PER_CTA = 4;

template <typename T>
struct DiagRowsArgs {
  using C = typename CT<T>::type;
  const C* in;
  C* out;
  long long rows, cols;
  const unsigned* rstr;
  const unsigned* cstr;
  const void* col_table;  // PHASE: C exp(i F_C); COEF: T F_C
  double rsame[FFGB_MAXN][FFGB_MAXN];
  double cross[FFGB_MAXN][FFGB_MAXN];
  int norb, zrep, mode, accumulate;
  double* partials;  // COEF only: when set, sum f |in|^2 per CTA here instead of writing out
  // when both are set the input is the outer product outer_row[r] * outer_col[c]
  // (a product state, e.g. a rotated Hartree-Fock state) and `in` is not read
  const C* outer_row;
  const C* outer_col;
  // stacked states (0: one state): each row holds ld columns, column c is
  // string c mod col_period, and columns whose index is >= cols (zero
  // padding) read the last string's entries
  long long ld, col_period;
};

// Per row, the row term and the cross term are tabulated over the two halves
// of the column string's bits: with h = norb / 2,
//   F(r) + sum_{l in occ(c)} w m_l(r) = L_r[c & (2^h - 1)] + H_r[c >> h]
// (w = -2 in the Z representation, else 1), each entry summed in FP64.  PHASE
// tables hold exp(i L), exp(i H); COEF tables the real sums.  An element then
// costs two shared-memory reads and two or three complex products instead of
// a loop over its occupied orbitals and a sine/cosine.
constexpr int DIAG_HALF = 1 << ((FFGB_MAXN + 1) / 2);

template <typename T>
__global__ void __launch_bounds__(DIAG_THREADS) diag_rows_kernel(const __grid_constant__ DiagRowsArgs<T> A) {
  using C = typename CT<T>::type;
  __shared__ double sm[FFGB_MAXN];
  __shared__ double sF;
  __shared__ C tl[DIAG_HALF], th[DIAG_HALF];  // PHASE tables
  __shared__ T ul[DIAG_HALF], uh[DIAG_HALF];  // COEF tables
  __shared__ double sred[DIAG_THREADS / 32];
  const int tid = threadIdx.x;
  const int h = A.norb / 2, nl = 1 << h, nh = 1 << (A.norb - h);
  const unsigned lmask = (unsigned)nl - 1u;
  const bool phase = A.mode == DIAG_PHASE;
  double part = 0.0;
  const long long r0 = (long long)blockIdx.x * DIAG_ROWS_PER_CTA;
  const long long r1 = min(r0 + DIAG_ROWS_PER_CTA, A.rows);
  for (long long r = r0; r < r1; ++r) {
    const unsigned rs = A.rstr[r];
    if (tid < A.norb) {
      double m = 0.0;
      for (int i = 0; i < A.norb; ++i) {
        const double gi = A.zrep ? (((rs >> i) & 1u) ? -1.0 : 1.0) : (double)((rs >> i) & 1u);
        m += A.cross[i][tid] * gi;
      }
      sm[tid] = A.zrep ? -2.0 * m : m;
    }
    if (tid == 32) {
      double f = 0.0;
      for (int i = 0; i < A.norb; ++i) {
        const double gi = A.zrep ? (((rs >> i) & 1u) ? -1.0 : 1.0) : (double)((rs >> i) & 1u);
        if (gi == 0.0) continue;
        for (int i2 = i; i2 < A.norb; ++i2) {
          const double gj = A.zrep ? (((rs >> i2) & 1u) ? -1.0 : 1.0) : (double)((rs >> i2) & 1u);
          f += A.rsame[i][i2] * gi * gj;
        }
      }
      if (A.zrep)  // g_l(c) = 1 - 2 n_l(c): the constant part of the cross term
        for (int l = 0; l < A.norb; ++l) {
          double m = 0.0;
          for (int i = 0; i < A.norb; ++i) m += A.cross[i][l] * (((rs >> i) & 1u) ? -1.0 : 1.0);
          f += m;
        }
      sF = f;
    }
    __syncthreads();
    for (int e = tid; e < nl + nh; e += DIAG_THREADS) {
      const bool low = e < nl;
      const unsigned bits = low ? (unsigned)e : (unsigned)(e - nl);
      const int off = low ? 0 : h;
      double a = low ? sF : 0.0;
      for (unsigned b = bits; b; b &= b - 1) a += sm[off + __ffs(b) - 1];
      if (phase) {
        const C z = phase_of(a, (C*)nullptr);
        if (low) tl[e] = z; else th[e - nl] = z;
      } else {
        if (low) ul[e] = (T)a; else uh[e - nl] = (T)a;
      }
    }
    __syncthreads();
    const long long ld = A.col_period ? A.ld : A.cols;
    const C* xin = A.in + r * ld;
    C* xout = A.out + r * ld;
    const C orow = A.outer_row ? A.outer_row[r] : cmake<C>(0.0, 0.0);
    for (long long c0 = tid; c0 < ld; c0 += DIAG_THREADS) {
      const long long c = A.col_period ? min(c0 % A.col_period, A.cols - 1) : c0;
      const unsigned s = A.cstr[c];
      C v = A.outer_row ? cmul(orow, A.outer_col[c]) : xin[c0];
      if (!phase) {
        const T z = ul[s & lmask] + uh[s >> h] + ((const T*)A.col_table)[c];
        if (A.partials) {
          part += (double)(z * (v.x * v.x + v.y * v.y));
          continue;
        }
        v.x *= z;
        v.y *= z;
      } else {
        v = cmul(cmul(v, ((const C*)A.col_table)[c]), cmul(tl[s & lmask], th[s >> h]));
      }
      if (A.accumulate) {
        C o = xout[c0];
        o.x += v.x;
        o.y += v.y;
        v = o;
      }
      xout[c0] = v;
    }
    __syncthreads();  // the next row overwrites the tables
  }
  if (A.partials) {  // fixed-order block reduction
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) sred[tid >> 5] = part;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < DIAG_THREADS / 32; ++w) t += sred[w];
      A.partials[blockIdx.x] = t;
    }
  }
}

// The occupied-orbital matrix of a rotated Hartree-Fock sector: for every
// string s (ascending occupied orbitals o_0 < ... < o_{n-1}) the amplitude of
// W(V) applied to the n lowest orbitals, det V[o_i][j] (i, j < n).  Gaussian
// elimination with partial pivoting in FP64, one string per thread; V is a
// kernel parameter (norb x norb complex, row-major).
struct SlaterMat {
  double v[FFGB_MAXN * FFGB_MAXN * 2];
};

template <typename C>
__global__ void __launch_bounds__(128) slater_dets_kernel(const unsigned* __restrict__ strings, long long dim,
                                                          int norb, int n, const __grid_constant__ SlaterMat V,
                                                          C* __restrict__ out) {
  const long long t = blockIdx.x * 128LL + threadIdx.x;
  if (t >= dim) return;
  const unsigned s = strings[t];
  double mr[FFGB_MAXN][FFGB_MAXN], mi[FFGB_MAXN][FFGB_MAXN];
  int row = 0;
  for (int o = 0; o < norb && row < n; ++o) {
    if (!((s >> o) & 1u)) continue;
    for (int j = 0; j < n; ++j) {
      mr[row][j] = V.v[2 * (o * norb + j)];
      mi[row][j] = V.v[2 * (o * norb + j) + 1];
    }
    ++row;
  }
  double dr = 1.0, di = 0.0;
  for (int k = 0; k < n; ++k) {
    int piv = k;
    double best = mr[k][k] * mr[k][k] + mi[k][k] * mi[k][k];
    for (int r = k + 1; r < n; ++r) {
      const double a = mr[r][k] * mr[r][k] + mi[r][k] * mi[r][k];
      if (a > best) {
        best = a;
        piv = r;
      }
    }
    if (piv != k) {
      for (int j = 0; j < n; ++j) {
        const double xr = mr[k][j], xi = mi[k][j];
        mr[k][j] = mr[piv][j];
        mi[k][j] = mi[piv][j];
        mr[piv][j] = xr;
        mi[piv][j] = xi;
      }
      dr = -dr;
      di = -di;
    }
    const double pr = mr[k][k], pi = mi[k][k];
    const double nr = dr * pr - di * pi, ni = dr * pi + di * pr;
    dr = nr;
    di = ni;
    if (best == 0.0) break;
    const double inv = 1.0 / best;  // 1 / p = conj(p) / |p|^2
    const double ir = pr * inv, ii = -pi * inv;
    for (int r = k + 1; r < n; ++r) {
      const double fr = mr[r][k] * ir - mi[r][k] * ii, fi = mr[r][k] * ii + mi[r][k] * ir;
      for (int j = k + 1; j < n; ++j) {
        mr[r][j] -= fr * mr[k][j] - fi * mi[k][j];
        mi[r][j] -= fr * mi[k][j] + fi * mr[k][j];
      }
    }
  }
  out[t] = cmake<C>(dr, di);
}

// x[r][c] *= row_ph[r] * col_ph[c] (either table optional).
template <typename C>
__global__ void __launch_bounds__(256) outer_scale_kernel(C* __restrict__ x, long long rows, long long cols,
                                                           const C* __restrict__ row_ph,
                                                           const C* __restrict__ col_ph) {
  const long long n = rows * cols;
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < n; i += (long long)gridDim.x * 256) {
    const long long r = i / cols, c = i - r * cols;
    C v = x[i];
    if (row_ph) v = cmul(v, row_ph[r]);
    if (col_ph) v = cmul(v, col_ph[c]);
    x[i] = v;
  }
}

}  // namespace ffgb
