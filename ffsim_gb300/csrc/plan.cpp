// Host-side planning of orbital rotations (see plan.h).
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace ffgb {

namespace {

inline cd at(const std::vector<cd>& m, int n, int r, int c) { return m[(size_t)r * n + c]; }

// One-sided (Hestenes) Jacobi sweeps on the columns of G (m x n, row-major):
// rotates column pairs until they are mutually orthogonal, accumulating the
// rotations into Y (n x n, G_out = G_in Y when Y starts as the identity).
// Accuracy is relative to each column's norm, so singular values spanning
// many orders of magnitude are all resolved.
void jacobi_columns(int m, int n, std::vector<cd>& G, std::vector<cd>& Y) {
  for (int sweep = 0; sweep < 80; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        double alpha = 0, beta = 0;
        cd gamma = 0;
        for (int k = 0; k < m; ++k) {
          cd gp = G[(size_t)k * n + p], gq = G[(size_t)k * n + q];
          alpha += std::norm(gp);
          beta += std::norm(gq);
          gamma += std::conj(gp) * gq;
        }
        double ag = std::abs(gamma);
        if (alpha == 0.0 || beta == 0.0 || ag <= 1e-17 * std::sqrt(alpha * beta)) continue;
        off = std::max(off, ag / std::sqrt(alpha * beta));
        double zeta = (beta - alpha) / (2.0 * ag);
        double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        cd e = std::conj(gamma / ag);  // e^{-i theta}
        for (int k = 0; k < m; ++k) {
          cd gp = G[(size_t)k * n + p], gq = G[(size_t)k * n + q];
          G[(size_t)k * n + p] = c * gp - s * e * gq;
          G[(size_t)k * n + q] = s * gp + c * e * gq;
        }
        for (int k = 0; k < n; ++k) {
          cd wp = Y[(size_t)k * n + p], wq = Y[(size_t)k * n + q];
          Y[(size_t)k * n + p] = c * wp - s * e * wq;
          Y[(size_t)k * n + q] = s * wp + c * e * wq;
        }
      }
    }
    if (off < 1e-16) break;
  }
}

// One-sided (Hestenes) Jacobi SVD of a square n x n matrix A (row-major):
// A = U diag(S) W^H, S descending.  Columns of U belonging to zero singular
// values are completed to an orthonormal basis.
void svd_jacobi(int n, const std::vector<cd>& A, std::vector<cd>& U, std::vector<double>& S,
                std::vector<cd>& W) {
  std::vector<cd> G = A;
  W.assign((size_t)n * n, cd(0));
  for (int i = 0; i < n; ++i) W[(size_t)i * n + i] = 1.0;
  jacobi_columns(n, n, G, W);
  S.assign(n, 0.0);
  for (int p = 0; p < n; ++p) {
    double ss = 0;
    for (int k = 0; k < n; ++k) ss += std::norm(G[(size_t)k * n + p]);
    S[p] = std::sqrt(ss);
  }
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return S[a] > S[b]; });
  std::vector<cd> U2((size_t)n * n, cd(0)), W2((size_t)n * n, cd(0));
  std::vector<double> S2(n);
  std::vector<bool> have(n, false);
  for (int j = 0; j < n; ++j) {
    int p = order[j];
    S2[j] = S[p];
    for (int k = 0; k < n; ++k) W2[(size_t)k * n + j] = W[(size_t)k * n + p];
    if (S[p] > 1e-300) {
      for (int k = 0; k < n; ++k) U2[(size_t)k * n + j] = G[(size_t)k * n + p] / S[p];
      have[j] = true;
    }
  }
  // complete missing columns by Gram-Schmidt on unit vectors
  for (int j = 0; j < n; ++j) {
    if (have[j]) continue;
    for (int e = 0; e < n; ++e) {
      std::vector<cd> v(n, cd(0));
      v[e] = 1.0;
      for (int pass = 0; pass < 2; ++pass)
        for (int o = 0; o < n; ++o) {
          if (!have[o]) continue;
          cd d = 0;
          for (int k = 0; k < n; ++k) d += std::conj(U2[(size_t)k * n + o]) * v[k];
          for (int k = 0; k < n; ++k) v[k] -= d * U2[(size_t)k * n + o];
        }
      double nv = 0;
      for (int k = 0; k < n; ++k) nv += std::norm(v[k]);
      nv = std::sqrt(nv);
      if (nv > 0.5) {
        for (int k = 0; k < n; ++k) U2[(size_t)k * n + j] = v[k] / nv;
        have[j] = true;
        break;
      }
    }
  }
  U.swap(U2);
  W.swap(W2);
  S.swap(S2);
}

// Householder QR of Z (m x n, m >= n, row-major): Z = Q R, Q m x m unitary.
void householder_qr(int m, int n, const std::vector<cd>& Z, std::vector<cd>& Q, std::vector<cd>& R) {
  R = Z;
  Q.assign((size_t)m * m, cd(0));
  for (int i = 0; i < m; ++i) Q[(size_t)i * m + i] = 1.0;
  std::vector<cd> v(m);
  for (int j = 0; j < n && j < m; ++j) {
    double nx = 0;
    for (int k = j; k < m; ++k) nx += std::norm(R[(size_t)k * n + j]);
    nx = std::sqrt(nx);
    if (nx == 0.0) continue;
    cd x0 = R[(size_t)j * n + j];
    cd ph = std::abs(x0) > 0 ? x0 / std::abs(x0) : cd(1.0);
    cd alpha = -ph * nx;
    double vn = 0;
    for (int k = j; k < m; ++k) {
      v[k] = R[(size_t)k * n + j];
      if (k == j) v[k] -= alpha;
      vn += std::norm(v[k]);
    }
    if (vn == 0.0) continue;
    // R <- (I - 2 v v^H / vn) R on rows j..m-1
    for (int c = j; c < n; ++c) {
      cd d = 0;
      for (int k = j; k < m; ++k) d += std::conj(v[k]) * R[(size_t)k * n + c];
      d *= 2.0 / vn;
      for (int k = j; k < m; ++k) R[(size_t)k * n + c] -= d * v[k];
    }
    // Q <- Q (I - 2 v v^H / vn) on columns j..m-1
    for (int r = 0; r < m; ++r) {
      cd d = 0;
      for (int k = j; k < m; ++k) d += Q[(size_t)r * m + k] * v[k];
      d *= 2.0 / vn;
      for (int k = j; k < m; ++k) Q[(size_t)r * m + k] -= d * std::conj(v[k]);
    }
  }
}

}  // namespace

void triangle_order(int b, std::vector<int>& l) {
  l.clear();
  for (int r = 0; r < b - 1; ++r)
    for (int col = b - 1; col > r; --col) l.push_back(col - 1);
}

void triangle_decompose(int b, const cd* X, std::vector<Givens>& rots, std::vector<cd>& diag) {
  std::vector<cd> M(X, X + (size_t)b * b);
  rots.clear();
  for (int r = 0; r < b - 1; ++r) {
    for (int col = b - 1; col > r; --col) {
      cd a = M[(size_t)r * b + col - 1], bb = M[(size_t)r * b + col];
      double aa = std::abs(a), rho = std::hypot(aa, std::abs(bb));
      double c = 1.0;
      cd s = 0.0;
      if (rho > 0.0) {
        cd ph = aa > 0 ? a / aa : cd(1.0);
        c = aa / rho;
        s = bb * std::conj(ph) / rho;
      }
      for (int row = 0; row < b; ++row) {
        cd x = M[(size_t)row * b + col - 1], y = M[(size_t)row * b + col];
        M[(size_t)row * b + col - 1] = c * x + std::conj(s) * y;
        M[(size_t)row * b + col] = -s * x + c * y;
      }
      rots.push_back({c, s});
    }
  }
  diag.resize(b);
  for (int i = 0; i < b; ++i) diag[i] = M[(size_t)i * b + i];
}

void brick_order(int b, std::vector<int>& l) {
  l.clear();
  for (int t = 0; t < b; ++t)
    for (int a = t % 2; a + 1 < b; a += 2) l.push_back(a);
}

// Rectangular ("brick") network: b layers alternating the pairs (0,1),(2,3),...
// and (1,2),(3,4),...  Built by nulling the entries of X alternately with
// column operations from the right and row operations from the left, then
// moving the left operations through the resulting diagonal (Clements et al.,
// Optica 3, 1460 (2016)), for the rotation form [[c, s], [-conj(s), c]].
bool brick_decompose(int b, const cd* X, std::vector<Givens>& rots, std::vector<cd>& diag) {
  std::vector<cd> U(X, X + (size_t)b * b);
  struct Op {
    int a;
    double c;
    cd s;
  };
  std::vector<Op> right, left;
  for (int i = 1; i < b; ++i) {
    if (i % 2 == 1) {
      for (int j = 0; j < i; ++j) {
        const int r = b - 1 - j, a = i - 1 - j;
        // column operation G^dag on (a, a+1): col_a <- c col_a + conj(s) col_{a+1}, zeroing U[r][a]
        const cd ua = U[(size_t)r * b + a], ub = U[(size_t)r * b + a + 1];
        const double rho = std::hypot(std::abs(ua), std::abs(ub));
        double c = 1.0;
        cd s = 0.0;
        if (rho > 0.0) {
          if (std::abs(ub) == 0.0) {
            c = 0.0;
            s = std::conj(-ua / std::abs(ua));
          } else {
            c = std::abs(ub) / rho;
            s = std::conj(-c * ua / ub);
          }
        }
        for (int row = 0; row < b; ++row) {
          const cd x = U[(size_t)row * b + a], y = U[(size_t)row * b + a + 1];
          U[(size_t)row * b + a] = c * x + std::conj(s) * y;
          U[(size_t)row * b + a + 1] = -s * x + c * y;
        }
        right.push_back({a, c, s});
      }
    } else {
      for (int j = 1; j <= i; ++j) {
        const int a = b + j - i - 2, col = j - 1;
        // row operation G on (a, a+1): row_{a+1} <- -conj(s) row_a + c row_{a+1}, zeroing U[a+1][col]
        const cd ua = U[(size_t)a * b + col], ub = U[(size_t)(a + 1) * b + col];
        const double rho = std::hypot(std::abs(ua), std::abs(ub));
        double c = 1.0;
        cd s = 0.0;
        if (rho > 0.0) {
          if (std::abs(ua) == 0.0) {
            c = 0.0;
            s = std::conj(ub / std::abs(ub));
          } else {
            c = std::abs(ua) / rho;
            s = std::conj(c * ub / ua);
          }
        }
        for (int cc = 0; cc < b; ++cc) {
          const cd x = U[(size_t)a * b + cc], y = U[(size_t)(a + 1) * b + cc];
          U[(size_t)a * b + cc] = c * x + s * y;
          U[(size_t)(a + 1) * b + cc] = -std::conj(s) * x + c * y;
        }
        left.push_back({a, c, s});
      }
    }
  }
  diag.resize(b);
  for (int i = 0; i < b; ++i) diag[i] = U[(size_t)i * b + i];
  // X = D * (left ops, inverted and moved through D) * (right ops, inverted), applied right to left
  std::vector<Op> seq(right.begin(), right.end());
  for (auto it = left.rbegin(); it != left.rend(); ++it) {
    const cd d1 = diag[it->a], d2 = diag[it->a + 1];
    seq.push_back({it->a, it->c, -it->s * d2 / d1});
  }
  // layer of every rotation (as early as its orbitals allow), then layer order
  std::vector<int> last(b, -1), layer(seq.size());
  for (size_t k = 0; k < seq.size(); ++k) {
    const int t = std::max(last[seq[k].a], last[seq[k].a + 1]) + 1;
    last[seq[k].a] = last[seq[k].a + 1] = t;
    layer[k] = t;
  }
  std::vector<size_t> idx(seq.size());
  for (size_t k = 0; k < idx.size(); ++k) idx[k] = k;
  std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) {
    return layer[x] != layer[y] ? layer[x] < layer[y] : seq[x].a < seq[y].a;
  });
  std::vector<int> want;
  brick_order(b, want);
  if (want.size() != seq.size()) return false;
  rots.clear();
  for (size_t k = 0; k < idx.size(); ++k) {
    const Op& o = seq[idx[k]];
    if (o.a != want[k]) return false;
    rots.push_back({o.c, o.s});
  }
  return true;
}

bool csd(int n, int h, const cd* Vp, std::vector<cd>& A1, std::vector<cd>& A2,
         std::vector<double>& cosv, std::vector<double>& sinv, std::vector<cd>& B1,
         std::vector<cd>& B2, double tol, double* err) {
  const int q = n - h;
  if (h < 1 || q < h) return false;
  std::vector<cd> V(Vp, Vp + (size_t)n * n);
  std::vector<cd> V11((size_t)h * h), V12((size_t)h * q), V21((size_t)q * h), V22((size_t)q * q);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      cd v = V[(size_t)r * n + c];
      if (r < h && c < h) V11[(size_t)r * h + c] = v;
      else if (r < h) V12[(size_t)r * q + (c - h)] = v;
      else if (c < h) V21[(size_t)(r - h) * h + c] = v;
      else V22[(size_t)(r - h) * q + (c - h)] = v;
    }
  std::vector<cd> U1, W1;
  std::vector<double> cs;
  svd_jacobi(h, V11, U1, cs, W1);
  // Cosines within rounding of 1 hide their sines (c = 1 - s^2/2), so V11's
  // right singular vectors are arbitrary inside that cluster; banded unitaries
  // (short-time evolutions, lattice hoppings) have many such sines between
  // 1e-16 and 1e-2.  For the columns with c > 1/sqrt(2) the right vectors are
  // re-resolved from V21 (Jacobi on V21 W_L, whose column norms are the sines)
  // and U1, c recomputed from V11 W_L, whose columns are then orthogonal.
  int nl = 0;
  while (nl < h && cs[nl] > 0.70710678118654752) ++nl;  // cs is descending
  if (nl > 1) {
    std::vector<cd> ZL((size_t)q * nl, cd(0)), Y((size_t)nl * nl, cd(0));
    for (int r = 0; r < q; ++r)
      for (int c = 0; c < nl; ++c) {
        cd acc = 0;
        for (int k = 0; k < h; ++k) acc += V21[(size_t)r * h + k] * W1[(size_t)k * h + c];
        ZL[(size_t)r * nl + c] = acc;
      }
    for (int i = 0; i < nl; ++i) Y[(size_t)i * nl + i] = 1.0;
    jacobi_columns(q, nl, ZL, Y);
    std::vector<cd> WL((size_t)h * nl, cd(0));
    for (int r = 0; r < h; ++r)
      for (int c = 0; c < nl; ++c) {
        cd acc = 0;
        for (int k = 0; k < nl; ++k) acc += W1[(size_t)r * h + k] * Y[(size_t)k * nl + c];
        WL[(size_t)r * nl + c] = acc;
      }
    for (int r = 0; r < h; ++r)
      for (int c = 0; c < nl; ++c) W1[(size_t)r * h + c] = WL[(size_t)r * nl + c];
    for (int c = 0; c < nl; ++c) {
      std::vector<cd> x(h, cd(0));
      for (int r = 0; r < h; ++r)
        for (int k = 0; k < h; ++k) x[r] += V11[(size_t)r * h + k] * W1[(size_t)k * h + c];
      double nx = 0;
      for (int r = 0; r < h; ++r) nx += std::norm(x[r]);
      nx = std::sqrt(nx);
      cs[c] = nx;
      for (int r = 0; r < h; ++r) U1[(size_t)r * h + c] = x[r] / nx;
    }
    // two Gram-Schmidt passes keep U1 unitary to rounding (the columns are
    // orthogonal in exact arithmetic, and their norms are at least 1/sqrt(2))
    for (int pass = 0; pass < 2; ++pass)
      for (int c = 0; c < nl; ++c) {
        for (int o = 0; o < h; ++o) {
          if (o == c || (o < nl && o > c)) continue;
          cd d = 0;
          for (int r = 0; r < h; ++r) d += std::conj(U1[(size_t)r * h + o]) * U1[(size_t)r * h + c];
          for (int r = 0; r < h; ++r) U1[(size_t)r * h + c] -= d * U1[(size_t)r * h + o];
        }
        double nu = 0;
        for (int r = 0; r < h; ++r) nu += std::norm(U1[(size_t)r * h + c]);
        nu = std::sqrt(nu);
        for (int r = 0; r < h; ++r) U1[(size_t)r * h + c] /= nu;
      }
  }
  // Z = V21 W1 (q x h)
  std::vector<cd> Z((size_t)q * h, cd(0));
  for (int r = 0; r < q; ++r)
    for (int c = 0; c < h; ++c) {
      cd acc = 0;
      for (int k = 0; k < h; ++k) acc += V21[(size_t)r * h + k] * W1[(size_t)k * h + c];
      Z[(size_t)r * h + c] = acc;
    }
  // QR in order of descending column norm (the sines): a column whose norm is
  // at rounding level has an arbitrary direction, and taken early its
  // reflection would move part of a larger later column off the diagonal of R.
  // The pairs (i, h + i) are independent, so permuting the index i of U1, W1
  // and the cosines together leaves the factorization intact.
  {
    std::vector<double> zn(h, 0.0);
    for (int c = 0; c < h; ++c)
      for (int r = 0; r < q; ++r) zn[c] += std::norm(Z[(size_t)r * h + c]);
    std::vector<int> order(h);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return zn[a] > zn[b]; });
    auto permute_cols = [&](std::vector<cd>& M, int rows) {
      std::vector<cd> T(M);
      for (int r = 0; r < rows; ++r)
        for (int c = 0; c < h; ++c) M[(size_t)r * h + c] = T[(size_t)r * h + order[c]];
    };
    permute_cols(Z, q);
    permute_cols(W1, h);
    permute_cols(U1, h);
    std::vector<double> cs2(h);
    for (int c = 0; c < h; ++c) cs2[c] = cs[order[c]];
    cs.swap(cs2);
  }
  std::vector<cd> Q, R;
  householder_qr(q, h, Z, Q, R);
  std::vector<cd> U2 = Q;
  std::vector<double> sn(h);
  for (int i = 0; i < h; ++i) {
    cd rii = R[(size_t)i * h + i];
    double ar = std::abs(rii);
    cd ph = ar > 0 ? rii / ar : cd(1.0);
    sn[i] = ar;
    for (int k = 0; k < q; ++k) U2[(size_t)k * q + i] *= ph;
  }
  cosv.resize(h);
  sinv.resize(h);
  for (int i = 0; i < h; ++i) {
    double th = std::atan2(sn[i], std::min(1.0, std::max(0.0, cs[i])));
    cosv[i] = std::cos(th);
    sinv[i] = std::sin(th);
  }
  // W2^H: rows i<h: c_i (U2^H V22)_i - s_i (U1^H V12)_i ; rows i>=h: (U2^H V22)_i
  std::vector<cd> P((size_t)q * q, cd(0)), K((size_t)h * q, cd(0));
  for (int r = 0; r < q; ++r)
    for (int c = 0; c < q; ++c) {
      cd acc = 0;
      for (int k = 0; k < q; ++k) acc += std::conj(U2[(size_t)k * q + r]) * V22[(size_t)k * q + c];
      P[(size_t)r * q + c] = acc;
    }
  for (int r = 0; r < h; ++r)
    for (int c = 0; c < q; ++c) {
      cd acc = 0;
      for (int k = 0; k < h; ++k) acc += std::conj(U1[(size_t)k * h + r]) * V12[(size_t)k * q + c];
      K[(size_t)r * q + c] = acc;
    }
  B2.assign((size_t)q * q, cd(0));
  for (int r = 0; r < q; ++r)
    for (int c = 0; c < q; ++c)
      B2[(size_t)r * q + c] = r < h ? cosv[r] * P[(size_t)r * q + c] - sinv[r] * K[(size_t)r * q + c]
                                    : P[(size_t)r * q + c];
  B1.assign((size_t)h * h, cd(0));
  for (int r = 0; r < h; ++r)
    for (int c = 0; c < h; ++c) B1[(size_t)r * h + c] = std::conj(W1[(size_t)c * h + r]);
  A1 = U1;
  A2 = U2;
  // reconstruction check
  std::vector<cd> CSB((size_t)n * n, cd(0));  // CS * diag(B1, B2)
  auto Bfull = [&](int r, int c) -> cd {
    if (r < h && c < h) return B1[(size_t)r * h + c];
    if (r >= h && c >= h) return B2[(size_t)(r - h) * q + (c - h)];
    return 0.0;
  };
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      cd acc;
      if (r < h) acc = cosv[r] * Bfull(r, c) - sinv[r] * Bfull(h + r, c);
      else if (r < 2 * h) acc = sinv[r - h] * Bfull(r - h, c) + cosv[r - h] * Bfull(r, c);
      else acc = Bfull(r, c);
      CSB[(size_t)r * n + c] = acc;
    }
  double e = 0;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      cd acc = 0;
      if (r < h)
        for (int k = 0; k < h; ++k) acc += A1[(size_t)r * h + k] * CSB[(size_t)k * n + c];
      else
        for (int k = 0; k < q; ++k) acc += A2[(size_t)(r - h) * q + k] * CSB[(size_t)(h + k) * n + c];
      e = std::max(e, std::abs(acc - V[(size_t)r * n + c]));
    }
  if (err) *err = e;
  return e <= tol;
}

namespace {
// multiply out a triangle network + diag into a b x b matrix (for checks)
// D * G_M ... G_1 for rotations G_k on (l_k, l_k + 1)
std::vector<cd> network_matrix(int b, const std::vector<Givens>& rots, const std::vector<int>& l,
                               const std::vector<cd>& diag) {
  std::vector<cd> M((size_t)b * b, cd(0));
  for (int i = 0; i < b; ++i) M[(size_t)i * b + i] = 1.0;
  for (size_t k = 0; k < rots.size(); ++k) {
    int a = l[k];
    double c = rots[k].c;
    cd s = rots[k].s;
    for (int col = 0; col < b; ++col) {
      cd x = M[(size_t)a * b + col], y = M[(size_t)(a + 1) * b + col];
      M[(size_t)a * b + col] = c * x + s * y;
      M[(size_t)(a + 1) * b + col] = -std::conj(s) * x + c * y;
    }
  }
  for (int r = 0; r < b; ++r)
    for (int col = 0; col < b; ++col) M[(size_t)r * b + col] *= diag[r];
  return M;
}

std::vector<cd> triangle_matrix(int b, const std::vector<Givens>& rots, const std::vector<cd>& diag) {
  std::vector<int> l;
  triangle_order(b, l);
  return network_matrix(b, rots, l, diag);
}

std::vector<cd> brick_matrix(int b, const std::vector<Givens>& rots, const std::vector<cd>& diag) {
  std::vector<int> l;
  brick_order(b, l);
  return network_matrix(b, rots, l, diag);
}
}  // namespace

// X (n x n, 8 < n <= 12) on orbitals [lo, lo + n) as three overlapping
// windows of 8: X = diag(1, A) * diag(B, 1) * diag(1, C), A and C on the last
// eight orbitals, B on the first eight (the last stage then never starts at
// orbital 0).  With t = n - 8 head orbitals: A^dag maps the last-eight-row part
// of the t head columns into the rows [t, 2t) (a QR factorization), which lie
// inside B's window when t <= 4; B^dag then maps the head columns onto unit
// vectors, so B^dag A^dag X = diag(1, C).  Each window's phases are pushed into
// the next window (the ones outside a window commute with it); d gets the rest.
bool three_windows(int n, const cd* X, int lo, std::vector<StageOp>& ops, std::vector<cd>& d) {
  const int t = n - 8;
  if (t < 1 || t > 4) return false;
  std::vector<cd> Y(X, X + (size_t)n * n);
  auto left_apply_dag = [&](const std::vector<cd>& U, int r0) {  // rows [r0, r0 + 8) of Y <- U^dag rows
    std::vector<cd> tmp((size_t)8 * n, cd(0));
    for (int r = 0; r < 8; ++r)
      for (int k = 0; k < 8; ++k) {
        const cd u = std::conj(U[(size_t)k * 8 + r]);
        if (u == cd(0)) continue;
        for (int c = 0; c < n; ++c) tmp[(size_t)r * n + c] += u * Y[(size_t)(r0 + k) * n + c];
      }
    std::copy(tmp.begin(), tmp.end(), Y.begin() + (size_t)r0 * n);
  };
  // A: Q^dag Z = R, nonzero in its first t rows
  std::vector<cd> Z((size_t)8 * t), A, R;
  for (int r = 0; r < 8; ++r)
    for (int c = 0; c < t; ++c) Z[(size_t)r * t + c] = Y[(size_t)(t + r) * n + c];
  householder_qr(8, t, Z, A, R);
  left_apply_dag(A, t);
  // B = [W | complement of W], W = rows [0, 8) of the head columns (orthonormal)
  std::vector<cd> Wm((size_t)8 * t), Q2, R2;
  for (int r = 0; r < 8; ++r)
    for (int c = 0; c < t; ++c) Wm[(size_t)r * t + c] = Y[(size_t)r * n + c];
  householder_qr(8, t, Wm, Q2, R2);
  std::vector<cd> B((size_t)64);
  for (int r = 0; r < 8; ++r) {
    for (int c = 0; c < t; ++c) B[(size_t)r * 8 + c] = Wm[(size_t)r * t + c];
    for (int c = t; c < 8; ++c) B[(size_t)r * 8 + c] = Q2[(size_t)r * 8 + c];
  }
  left_apply_dag(B, 0);
  // Y = diag(1, C) now
  double off = 0;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      if (r < t || c < t) off = std::max(off, std::abs(Y[(size_t)r * n + c] - (r == c ? cd(1) : cd(0))));
  if (off > 1e-10) return false;
  std::vector<cd> C((size_t)64);
  for (int r = 0; r < 8; ++r)
    for (int c = 0; c < 8; ++c) C[(size_t)r * 8 + c] = Y[(size_t)(t + r) * n + t + c];
  StageOp wc, wb, wa;
  wc.type = wb.type = wa.type = 0;
  wc.b = wb.b = wa.b = 8;
  wc.lo = wa.lo = lo + t;
  wb.lo = lo;
  std::vector<cd> dC, dB, dA;
  if (!brick_decompose(8, C.data(), wc.net, dC)) return false;
  for (int r = 0; r < 8; ++r)  // C's phases on orbitals [t, 8) into B's columns
    for (int c = t; c < 8; ++c) B[(size_t)r * 8 + c] *= dC[c - t];
  if (!brick_decompose(8, B.data(), wb.net, dB)) return false;
  for (int r = 0; r < 8; ++r)  // B's phases on [t, 8) and C's on [8, n) into A's columns
    for (int c = 0; c < 8; ++c) A[(size_t)r * 8 + c] *= t + c < 8 ? dB[t + c] : dC[c];
  if (!brick_decompose(8, A.data(), wa.net, dA)) return false;
  d.assign(n, cd(1));
  for (int i = 0; i < t; ++i) d[i] = dB[i];
  for (int i = t; i < n; ++i) d[i] = dA[i - t];
  ops.push_back(std::move(wc));
  ops.push_back(std::move(wb));
  ops.push_back(std::move(wa));
  return true;
}

// X (n x n, unitary) on orbitals [lo, lo + n) = diag(d) * (ops appended here,
// applied first to last).  Blocks of at most 8 orbitals are one window, of 9 to
// 12 orbitals three overlapping windows; larger blocks are split by a
// cosine-sine decomposition (halves of at most 8 orbitals up to 16, else 8
// plus the rest) whose right blocks' phases are pushed through the cross-half
// rotations into the left blocks.
bool block_ops(int n, const cd* X, int lo, std::vector<StageOp>& ops, std::vector<cd>& d) {
  if (n <= 8) {
    StageOp w;
    w.type = 0;
    w.lo = lo;
    w.b = n;
    if (!brick_decompose(n, X, w.net, d)) return false;
    ops.push_back(std::move(w));
    return true;
  }
  if (n <= 12) {
    const size_t mark = ops.size();
    if (three_windows(n, X, lo, ops, d)) return true;
    ops.resize(mark);
  }
  const int h = n <= 16 ? n / 2 : 8, q = n - h;
  std::vector<cd> A1, A2, B1, B2;
  std::vector<double> cv, sv;
  double err = 0;
  if (!csd(n, h, X, A1, A2, cv, sv, B1, B2, 1e-11, &err)) return false;
  std::vector<cd> dB1, dB2, dA1, dA2;
  if (!block_ops(h, B1.data(), lo, ops, dB1) || !block_ops(q, B2.data(), lo + h, ops, dB2)) return false;
  std::vector<cd> dB(dB1);
  dB.insert(dB.end(), dB2.begin(), dB2.end());
  StageOp c;
  c.type = 1;
  c.lo = lo;
  c.b = h;
  for (int i = 0; i < h; ++i) {
    const int j = h + i;
    Pair2 p;
    p.i = lo + i;
    p.j = lo + j;
    p.g00 = cv[i];
    p.g01 = std::conj(dB[i]) * (-sv[i]) * dB[j];
    p.g10 = std::conj(dB[j]) * sv[i] * dB[i];
    p.g11 = cv[i];
    c.pairs.push_back(p);
  }
  ops.push_back(std::move(c));
  for (int r = 0; r < h; ++r)
    for (int cc = 0; cc < h; ++cc) A1[(size_t)r * h + cc] *= dB1[cc];
  for (int r = 0; r < q; ++r)
    for (int cc = 0; cc < q; ++cc) A2[(size_t)r * q + cc] *= dB2[cc];
  if (!block_ops(h, A1.data(), lo, ops, dA1) || !block_ops(q, A2.data(), lo + h, ops, dA2)) return false;
  d = dA1;
  d.insert(d.end(), dA2.begin(), dA2.end());
  return true;
}

// diag(D) * (ops applied in order) as an n x n matrix.
std::vector<cd> ops_matrix(int n, const std::vector<StageOp>& ops, const std::vector<cd>& D) {
  std::vector<cd> M((size_t)n * n, cd(0));
  for (int i = 0; i < n; ++i) M[(size_t)i * n + i] = 1.0;
  auto rot = [&](int a, int b2, cd g00, cd g01, cd g10, cd g11) {
    for (int col = 0; col < n; ++col) {
      const cd x = M[(size_t)a * n + col], y = M[(size_t)b2 * n + col];
      M[(size_t)a * n + col] = g00 * x + g01 * y;
      M[(size_t)b2 * n + col] = g10 * x + g11 * y;
    }
  };
  for (const StageOp& op : ops) {
    if (op.type == 0) {
      std::vector<int> l;
      brick_order(op.b, l);
      for (size_t k = 0; k < op.net.size(); ++k) {
        const Givens& g = op.net[k];
        rot(op.lo + l[k], op.lo + l[k] + 1, g.c, g.s, -std::conj(g.s), g.c);
      }
    } else {
      for (const Pair2& p : op.pairs) rot(p.i, p.j, p.g00, p.g01, p.g10, p.g11);
    }
  }
  for (int r = 0; r < n; ++r)
    for (int col = 0; col < n; ++col) M[(size_t)r * n + col] *= D[r];
  return M;
}

bool plan_sector(int norb, const cd* V, bool want_csd, SectorPlan& plan) {
  plan = SectorPlan();
  plan.norb = norb;
  if (norb == 0) {
    plan.kind = PLAN_IDENTITY;
    return true;
  }
  if (!want_csd || norb > 18) {
    plan.kind = PLAN_TRIANGLE;
    triangle_decompose(norb, V, plan.tri, plan.diag);
    triangle_order(norb, plan.tri_l);
    std::vector<cd> M = triangle_matrix(norb, plan.tri, plan.diag);
    double e = 0;
    for (size_t i = 0; i < M.size(); ++i) e = std::max(e, std::abs(M[i] - V[i]));
    plan.max_err = e;
    return true;
  }
  if (norb <= 8) {
    plan.kind = PLAN_FULL;
    plan.h = norb;
    if (!brick_decompose(norb, V, plan.tri, plan.diag)) return plan_sector(norb, V, false, plan);
    brick_order(norb, plan.tri_l);
    std::vector<cd> M = brick_matrix(norb, plan.tri, plan.diag);
    double e = 0;
    for (size_t i = 0; i < M.size(); ++i) e = std::max(e, std::abs(M[i] - V[i]));
    plan.max_err = e;
    return true;
  }
  const int h = norb / 2, q = norb - h;
  if (q > 8) {  // nested blocks: the stage sequence only
    plan.kind = PLAN_CSD;
    plan.h = 8;
    if (!block_ops(norb, V, 0, plan.ops, plan.diag)) return plan_sector(norb, V, false, plan);
    std::vector<cd> M = ops_matrix(norb, plan.ops, plan.diag);
    double e = 0;
    for (size_t i = 0; i < M.size(); ++i) e = std::max(e, std::abs(M[i] - V[i]));
    plan.max_err = e;
    if (e > 1e-10) return plan_sector(norb, V, false, plan);
    return true;
  }
  std::vector<cd> A1, A2, B1, B2;
  std::vector<double> cv, sv;
  double err = 0;
  if (!csd(norb, h, V, A1, A2, cv, sv, B1, B2, 1e-11, &err)) {
    // fall back to the generic network
    return plan_sector(norb, V, false, plan);
  }
  plan.kind = PLAN_CSD;
  plan.h = h;
  std::vector<cd> dB1, dB2, dA1, dA2;
  if (!brick_decompose(h, B1.data(), plan.b1, dB1) || !brick_decompose(q, B2.data(), plan.b2, dB2))
    return plan_sector(norb, V, false, plan);
  std::vector<cd> dB(dB1);
  dB.insert(dB.end(), dB2.begin(), dB2.end());
  plan.cs.clear();
  for (int i = 0; i < h; ++i) {
    int j = h + i;
    Pair2 p;
    p.i = i;
    p.j = j;
    p.g00 = cv[i];
    p.g01 = std::conj(dB[i]) * (-sv[i]) * dB[j];
    p.g10 = std::conj(dB[j]) * sv[i] * dB[i];
    p.g11 = cv[i];
    plan.cs.push_back(p);
  }
  // A' = A diag(dB)
  for (int r = 0; r < h; ++r)
    for (int c = 0; c < h; ++c) A1[(size_t)r * h + c] *= dB1[c];
  for (int r = 0; r < q; ++r)
    for (int c = 0; c < q; ++c) A2[(size_t)r * q + c] *= dB2[c];
  if (!brick_decompose(h, A1.data(), plan.a1, dA1) || !brick_decompose(q, A2.data(), plan.a2, dA2))
    return plan_sector(norb, V, false, plan);
  plan.diag = dA1;
  plan.diag.insert(plan.diag.end(), dA2.begin(), dA2.end());
  // multiply the plan back out to measure its error
  std::vector<cd> TB1 = brick_matrix(h, plan.b1, std::vector<cd>(h, cd(1)));
  std::vector<cd> TB2 = brick_matrix(q, plan.b2, std::vector<cd>(q, cd(1)));
  std::vector<cd> TA1 = brick_matrix(h, plan.a1, dA1);
  std::vector<cd> TA2 = brick_matrix(q, plan.a2, dA2);
  auto blk = [&](const std::vector<cd>& X1, const std::vector<cd>& X2) {
    std::vector<cd> M((size_t)norb * norb, cd(0));
    for (int r = 0; r < h; ++r)
      for (int c = 0; c < h; ++c) M[(size_t)r * norb + c] = X1[(size_t)r * h + c];
    for (int r = 0; r < q; ++r)
      for (int c = 0; c < q; ++c) M[(size_t)(h + r) * norb + h + c] = X2[(size_t)r * q + c];
    return M;
  };
  std::vector<cd> MB = blk(TB1, TB2), MA = blk(TA1, TA2);
  std::vector<cd> MC((size_t)norb * norb, cd(0));
  for (int i = 0; i < norb; ++i) MC[(size_t)i * norb + i] = 1.0;
  for (const Pair2& p : plan.cs) {
    MC[(size_t)p.i * norb + p.i] = p.g00;
    MC[(size_t)p.i * norb + p.j] = p.g01;
    MC[(size_t)p.j * norb + p.i] = p.g10;
    MC[(size_t)p.j * norb + p.j] = p.g11;
  }
  auto mm = [&](const std::vector<cd>& X, const std::vector<cd>& Y) {
    std::vector<cd> Out((size_t)norb * norb, cd(0));
    for (int r = 0; r < norb; ++r)
      for (int k = 0; k < norb; ++k) {
        cd x = X[(size_t)r * norb + k];
        if (x == cd(0)) continue;
        for (int c = 0; c < norb; ++c) Out[(size_t)r * norb + c] += x * Y[(size_t)k * norb + c];
      }
    return Out;
  };
  std::vector<cd> full = mm(MA, mm(MC, MB));
  double e = 0;
  for (size_t i = 0; i < full.size(); ++i) e = std::max(e, std::abs(full[i] - V[i]));
  plan.max_err = e;
  if (e > 1e-10) return plan_sector(norb, V, false, plan);
  auto window = [](int lo, int b, const std::vector<Givens>& net) {
    StageOp w;
    w.type = 0;
    w.lo = lo;
    w.b = b;
    w.net = net;
    return w;
  };
  StageOp c;
  c.type = 1;
  c.lo = 0;
  c.b = h;
  c.pairs = plan.cs;
  plan.ops = {window(0, h, plan.b1), window(h, q, plan.b2), c, window(0, h, plan.a1), window(h, q, plan.a2)};
  plan.csd_diag = plan.diag;
  if (norb <= 12) {  // three windows instead of five stages
    std::vector<StageOp> ops3;
    std::vector<cd> d3;
    if (three_windows(norb, V, 0, ops3, d3)) {
      std::vector<cd> M = ops_matrix(norb, ops3, d3);
      double e3 = 0;
      for (size_t i = 0; i < M.size(); ++i) e3 = std::max(e3, std::abs(M[i] - V[i]));
      if (e3 <= 1e-10) {
        plan.ops = std::move(ops3);
        plan.diag = std::move(d3);
        plan.max_err = std::max(plan.max_err, e3);
      }
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// Reference Givens decomposition, restated (src/linalg/givens.rs:20-149)
// ---------------------------------------------------------------------------
namespace {
void zrotg_safe(cd a, cd b, double tol, double* c, cd* s) {
  double aa = std::abs(a), ab = std::abs(b);
  if (ab <= tol) {
    *c = 1.0;
    *s = 0.0;
    return;
  }
  if (aa <= tol) {
    *c = 0.0;
    *s = 1.0;
    return;
  }
  double r = std::hypot(aa, ab);
  *c = std::min(1.0, std::max(-1.0, aa / r));
  *s = (a / aa) * std::conj(b) / r;
}
}  // namespace

bool reference_givens_decomposition(int n, const cd* mat, double tol, std::vector<RefGivens>& rots,
                                    std::vector<cd>& diag) {
  std::vector<cd> m(mat, mat + (size_t)n * n);
  std::vector<RefGivens> left;
  rots.clear();
  auto rot_cols = [&](int x, int y, double c, cd s) {
    for (int r = 0; r < n; ++r) {
      cd xo = m[(size_t)r * n + x], yo = m[(size_t)r * n + y];
      m[(size_t)r * n + x] = c * xo + s * yo;
      m[(size_t)r * n + y] = c * yo - std::conj(s) * xo;
    }
  };
  auto rot_rows = [&](int x, int y, double c, cd s) {
    for (int col = 0; col < n; ++col) {
      cd xo = m[(size_t)x * n + col], yo = m[(size_t)y * n + col];
      m[(size_t)x * n + col] = c * xo + s * yo;
      m[(size_t)y * n + col] = c * yo - std::conj(s) * xo;
    }
  };
  for (int i = 0; i + 1 < n; ++i) {
    for (int j = 0; j <= i; ++j) {
      if (i % 2 == 0) {
        int t = i - j, row = n - j - 1;
        if (std::abs(m[(size_t)row * n + t]) > tol) {
          double c;
          cd s;
          zrotg_safe(m[(size_t)row * n + t + 1], m[(size_t)row * n + t], tol, &c, &s);
          rots.push_back({c, s, t + 1, t});
          rot_cols(t + 1, t, c, s);
        }
      } else {
        int t = n - i + j - 1, col = j;
        if (std::abs(m[(size_t)t * n + col]) > tol) {
          double c;
          cd s;
          zrotg_safe(m[(size_t)(t - 1) * n + col], m[(size_t)t * n + col], tol, &c, &s);
          left.push_back({c, s, t - 1, t});
          rot_rows(t - 1, t, c, s);
        }
      }
    }
  }
  for (auto it = left.rbegin(); it != left.rend(); ++it) {
    int i = it->i, j = it->j;
    double c;
    cd s;
    zrotg_safe(it->c * m[(size_t)j * n + j], std::conj(it->s) * m[(size_t)i * n + i], tol, &c, &s);
    rots.push_back({c, -std::conj(s), i, j});
    cd di = m[(size_t)i * n + i], dj = m[(size_t)j * n + j];
    cd g00 = c * di, g01 = -s * dj, g10 = std::conj(s) * di, g11 = c * dj;
    double cn;
    cd sn;
    zrotg_safe(g11, g10, tol, &cn, &sn);
    m[(size_t)i * n + i] = g00 * cn + g01 * (-std::conj(sn));
    m[(size_t)j * n + j] = g10 * sn + g11 * cn;
  }
  diag.resize(n);
  for (int i = 0; i < n; ++i) diag[i] = m[(size_t)i * n + i];
  return true;
}

// ---------------------------------------------------------------------------
// Hermitian eigendecomposition by cyclic complex Jacobi rotations
// ---------------------------------------------------------------------------
void hermitian_eigh(int n, const cd* Ap, std::vector<double>& w, std::vector<cd>& vecs) {
  std::vector<cd> A(Ap, Ap + (size_t)n * n);
  for (int r = 0; r < n; ++r) {  // symmetrize
    A[(size_t)r * n + r] = A[(size_t)r * n + r].real();
    for (int c = r + 1; c < n; ++c) {
      cd v = 0.5 * (A[(size_t)r * n + c] + std::conj(A[(size_t)c * n + r]));
      A[(size_t)r * n + c] = v;
      A[(size_t)c * n + r] = std::conj(v);
    }
  }
  vecs.assign((size_t)n * n, cd(0));
  for (int i = 0; i < n; ++i) vecs[(size_t)i * n + i] = 1.0;
  double scale = 0;
  for (auto& x : A) scale = std::max(scale, std::abs(x));
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off = std::max(off, std::abs(A[(size_t)p * n + q]));
    if (off <= 1e-16 * std::max(scale, 1e-300)) break;
    for (int p = 0; p < n; ++p) {
      for (int q = p + 1; q < n; ++q) {
        cd apq = A[(size_t)p * n + q];
        double a = std::abs(apq);
        if (a <= 1e-300) continue;
        cd e = apq / a;  // e^{i phi}
        double app = A[(size_t)p * n + p].real(), aqq = A[(size_t)q * n + q].real();
        double tau = (aqq - app) / (2.0 * a);
        double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
        // J = [[c, s], [-s conj(e), c conj(e)]] on columns (p, q): A <- J^H A J
        cd j00 = c, j01 = s, j10 = -s * std::conj(e), j11 = c * std::conj(e);
        for (int k = 0; k < n; ++k) {  // A <- A J
          cd x = A[(size_t)k * n + p], y = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = x * j00 + y * j10;
          A[(size_t)k * n + q] = x * j01 + y * j11;
        }
        for (int k = 0; k < n; ++k) {  // A <- J^H A
          cd x = A[(size_t)p * n + k], y = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = std::conj(j00) * x + std::conj(j10) * y;
          A[(size_t)q * n + k] = std::conj(j01) * x + std::conj(j11) * y;
        }
        A[(size_t)p * n + q] = 0.0;
        A[(size_t)q * n + p] = 0.0;
        for (int k = 0; k < n; ++k) {
          cd x = vecs[(size_t)k * n + p], y = vecs[(size_t)k * n + q];
          vecs[(size_t)k * n + p] = x * j00 + y * j10;
          vecs[(size_t)k * n + q] = x * j01 + y * j11;
        }
      }
    }
  }
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::vector<double> d(n);
  for (int i = 0; i < n; ++i) d[i] = A[(size_t)i * n + i].real();
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return d[a] < d[b]; });
  w.resize(n);
  std::vector<cd> v2((size_t)n * n);
  for (int j = 0; j < n; ++j) {
    w[j] = d[order[j]];
    for (int k = 0; k < n; ++k) v2[(size_t)k * n + j] = vecs[(size_t)k * n + order[j]];
  }
  vecs.swap(v2);
}

}  // namespace ffgb
