// Host-side planning of orbital rotations for the sector kernels.
//
// An orbital rotation V (norb x norb unitary) acts on one spin sector as
// W(V), the representation a^dag_k -> sum_l V_lk a^dag_l.  W is a group
// homomorphism, so any exact factorization of V into simple unitaries gives
// W(V) as the product of their actions.  Two factorizations are planned:
//
//  * TRIANGLE: V = D * G_M ... G_1, adjacent Givens rotations G_k on (l, l+1)
//    in a fixed order (see triangle_decompose), applied one per shared-memory
//    sweep.  Used for complex128 and as the generic path.
//  * CSD (complex64, 9 <= norb <= 18): V = D * (T_A1 + T_A2) * CS' * (T_B1 + T_B2),
//    a cosine-sine decomposition over the halves [0,h) and [h,norb); each
//    half-block of at most 8 orbitals is a window network (brick_decompose)
//    applied in registers, one of 9 to 12 orbitals three overlapping windows
//    (three_windows); CS' is h commuting rotations on orbital pairs (i, h+i).
//    `ops` lists the stages of the stage kernels: three windows for
//    norb <= 12, five stages up to 16, nine for 17 and 18 (h = 8).  For
//    norb <= 16 the fields b1 .. a2, cs keep the five-stage form for the
//    sector kernel, with its phases in csd_diag.
//    For norb <= 8 the whole sector is one window ("FULL").
#pragma once

#include <complex>
#include <vector>

namespace ffgb {

using cd = std::complex<double>;

struct Givens {  // 2x2 block [[c, s], [-conj(s), c]] on orbitals (l, l+1)
  double c;
  cd s;
};

struct Pair2 {  // general 2x2 unitary block on orbitals (i, j), i < j
  int i, j;
  cd g00, g01, g10, g11;
};

enum PlanKind { PLAN_IDENTITY = 0, PLAN_TRIANGLE = 1, PLAN_FULL = 2, PLAN_CSD = 3 };

// One stage of a cosine-sine plan, in application order.
struct StageOp {
  int type = 0;  // 0: window network on orbitals [lo, lo + b); 1: cross-half rotations
  int lo = 0;    // first orbital
  int b = 0;     // window size, or the half width hh of the sites (lo + i, lo + hh + i), i < hh
  std::vector<Givens> net;   // window: brick network (brick_order)
  std::vector<Pair2> pairs;  // cross-half: pairs[i] on (lo + i, lo + hh + i)
};

struct SectorPlan {
  int kind = PLAN_IDENTITY;
  int norb = 0;
  int h = 0;  // split point for CSD; norb for FULL
  std::vector<Givens> tri;   // TRIANGLE / FULL network (norb(norb-1)/2)
  std::vector<int> tri_l;    // TRIANGLE: lower orbital of each rotation
  std::vector<Givens> b1, b2, a1, a2;  // CSD window networks (norb <= 16)
  std::vector<Pair2> cs;     // CSD middle rotations (i, h+i) (norb <= 16)
  std::vector<StageOp> ops;  // CSD: the stage sequence (every norb; blocks above 8 orbitals nested)
  std::vector<cd> diag;      // final per-orbital phases (norb); of `ops` for CSD plans
  std::vector<cd> csd_diag;  // CSD, norb <= 16: the phases of the five-stage form (b1 .. a2, cs)
  double max_err = 0.0;      // reconstruction error of the factorization
};

// Fixed triangular network: X (b x b unitary, row-major) = D * G_M ... G_1.
// Rotation k acts on local orbitals (l_k, l_k+1), l_k from triangle_order().
void triangle_decompose(int b, const cd* X, std::vector<Givens>& rots, std::vector<cd>& diag);
void triangle_order(int b, std::vector<int>& l);
// Rectangular network of b layers alternating the pairs (0,1),(2,3),... and
// (1,2),(3,4),...: X = D * (rotations in brick_order, applied first to last).
// Window networks use it (a loop of identical layer pairs).  False if the
// construction does not give the rectangular shape.
bool brick_decompose(int b, const cd* X, std::vector<Givens>& rots, std::vector<cd>& diag);
void brick_order(int b, std::vector<int>& l);

// Cosine-sine decomposition of V (n x n) at split h (h <= n-h <= h+1):
// V = diag(A1, A2) * CS * diag(B1, B2); returns false if it fails to
// reconstruct V within tol.
bool csd(int n, int h, const cd* V, std::vector<cd>& A1, std::vector<cd>& A2,
         std::vector<double>& cosv, std::vector<double>& sinv, std::vector<cd>& B1,
         std::vector<cd>& B2, double tol, double* err);

// X (n x n, 8 < n <= 12) on orbitals [lo, lo + n) = diag(d) * three windows of
// eight orbitals (appended to ops, applied first to last).
bool three_windows(int n, const cd* X, int lo, std::vector<StageOp>& ops, std::vector<cd>& d);
// diag(D) * (ops applied in order) as an n x n matrix.
std::vector<cd> ops_matrix(int n, const std::vector<StageOp>& ops, const std::vector<cd>& D);

// Build the plan for W(V) on a sector with nocc electrons in norb orbitals.
// want_csd selects the register-window factorization when norb allows it.
bool plan_sector(int norb, const cd* V, bool want_csd, SectorPlan& plan);

// Restatement of the reference Givens decomposition (src/linalg/givens.rs:68-149):
// U = D * G_L^* ... G_1^*, rotations (c, s, i, j).
struct RefGivens {
  double c;
  cd s;
  int i, j;
};
bool reference_givens_decomposition(int n, const cd* mat, double tol, std::vector<RefGivens>& rots,
                                    std::vector<cd>& diag);

// Hermitian eigendecomposition (cyclic complex Jacobi), ascending eigenvalues,
// eigenvectors as columns of vecs (row-major n x n).
void hermitian_eigh(int n, const cd* A, std::vector<double>& w, std::vector<cd>& vecs);

}  // namespace ffgb
