/*
 * CPU restatement of the reference's Rust kernels for the statevector gate
 * path -- TEST/BASELINE INFRASTRUCTURE ONLY (timed as the CPU baseline by
 * bench.py and used by tests as a second CPU checker; never by the product).
 *
 * The reference kernels (src/gates/*.rs, src/contract/*.rs) are Rust and
 * cannot be built here (no Rust toolchain).  This file restates them in C99
 * with OpenMP threads in place of rayon / std::thread::scope, keeping the
 * same data layout (row-major (dim_a, dim_b) complex128) and the same work
 * decomposition:
 *   ref_givens_rows      src/gates/orbital_rotation.rs:18-104 (row pairs, threads over pairs)
 *   ref_phase_rows       src/gates/phase_shift.rs:17-30
 *   ref_diag_coulomb_num src/gates/diag_coulomb.rs:19-90 (three-phase product)
 *   ref_num_op_sum_rows  src/gates/num_op_sum.rs:18-36
 *   ref_contract_dc_num  src/contract/diag_coulomb.rs:22-95
 *   ref_contract_nos_rows src/contract/num_op_sum.rs:20-39
 * Build: oracle/Makefile (gcc -O3 -fopenmp -shared).
 */
#include <complex.h>
#include <stdlib.h>
#include <string.h>

typedef double complex zd;

void ref_givens_rows(zd* vec, long dim_b, double c, double s_re, double s_im, const long* slice1,
                     const long* slice2, long n_pairs) {
  const zd s = s_re + I * s_im;
  const zd sc = conj(s);
#pragma omp parallel for schedule(static)
  for (long k = 0; k < n_pairs; ++k) {
    zd* ri = vec + slice1[k] * dim_b;
    zd* rj = vec + slice2[k] * dim_b;
    for (long q = 0; q < dim_b; ++q) {
      const zd a = ri[q], b = rj[q];
      ri[q] = c * a + s * b;
      rj[q] = c * b - sc * a;
    }
  }
}

void ref_phase_rows(zd* vec, long dim_b, double p_re, double p_im, const long* rows, long n_rows) {
  const zd p = p_re + I * p_im;
  for (long k = 0; k < n_rows; ++k) {
    zd* r = vec + rows[k] * dim_b;
    for (long q = 0; q < dim_b; ++q) r[q] *= p;
  }
}

/* mat_exp_*: norb*norb complex; occ_a: dim_a*n_alpha; occ_b: dim_b*n_beta */
void ref_diag_coulomb_num(zd* vec, long dim_a, long dim_b, int norb, const zd* eaa, const zd* eab,
                          const zd* ebb, const long* occ_a, int n_alpha, const long* occ_b, int n_beta) {
  zd* beta_ph = (zd*)malloc(sizeof(zd) * (size_t)dim_b);
  zd* alpha_ph = (zd*)malloc(sizeof(zd) * (size_t)dim_a);
  zd* phase_map = (zd*)malloc(sizeof(zd) * (size_t)dim_a * (size_t)norb);
#pragma omp parallel for schedule(static)
  for (long b = 0; b < dim_b; ++b) {
    zd ph = 1.0;
    const long* o = occ_b + b * n_beta;
    for (int j = 0; j < n_beta; ++j)
      for (int k = j; k < n_beta; ++k) ph *= ebb[o[j] * norb + o[k]];
    beta_ph[b] = ph;
  }
#pragma omp parallel for schedule(static)
  for (long a = 0; a < dim_a; ++a) {
    zd ph = 1.0;
    const long* o = occ_a + a * n_alpha;
    zd* row = phase_map + a * norb;
    for (int q = 0; q < norb; ++q) row[q] = 1.0;
    for (int j = 0; j < n_alpha; ++j) {
      for (int q = 0; q < norb; ++q) row[q] *= eab[o[j] * norb + q];
      for (int k = j; k < n_alpha; ++k) ph *= eaa[o[j] * norb + o[k]];
    }
    alpha_ph[a] = ph;
  }
#pragma omp parallel for schedule(static)
  for (long a = 0; a < dim_a; ++a) {
    const zd* pm = phase_map + a * norb;
    zd* row = vec + a * dim_b;
    for (long b = 0; b < dim_b; ++b) {
      zd ph = alpha_ph[a] * beta_ph[b];
      const long* o = occ_b + b * n_beta;
      for (int j = 0; j < n_beta; ++j) ph *= pm[o[j]];
      row[b] *= ph;
    }
  }
  free(beta_ph);
  free(alpha_ph);
  free(phase_map);
}

/* rows of vec (stride row_stride, elem_stride) scaled by prod phases[occ] */
void ref_num_op_sum_rows(zd* vec, long n_rows, long row_len, long row_stride, long elem_stride,
                         const zd* phases, const long* occ, int nocc) {
#pragma omp parallel for schedule(static)
  for (long r = 0; r < n_rows; ++r) {
    zd ph = 1.0;
    for (int j = 0; j < nocc; ++j) ph *= phases[occ[r * nocc + j]];
    zd* p = vec + r * row_stride;
    for (long q = 0; q < row_len; ++q) p[q * elem_stride] *= ph;
  }
}

void ref_contract_dc_num(const zd* vec, zd* out, long dim_a, long dim_b, int norb, const double* maa,
                         const double* mab, const double* mbb, const long* occ_a, int n_alpha,
                         const long* occ_b, int n_beta) {
  double* beta_c = (double*)malloc(sizeof(double) * (size_t)dim_b);
  double* alpha_c = (double*)malloc(sizeof(double) * (size_t)dim_a);
  double* cmap = (double*)calloc((size_t)dim_a * (size_t)norb, sizeof(double));
#pragma omp parallel for schedule(static)
  for (long b = 0; b < dim_b; ++b) {
    double c = 0.0;
    const long* o = occ_b + b * n_beta;
    for (int j = 0; j < n_beta; ++j)
      for (int k = j; k < n_beta; ++k) c += mbb[o[j] * norb + o[k]];
    beta_c[b] = c;
  }
#pragma omp parallel for schedule(static)
  for (long a = 0; a < dim_a; ++a) {
    double c = 0.0;
    const long* o = occ_a + a * n_alpha;
    double* row = cmap + a * norb;
    for (int j = 0; j < n_alpha; ++j) {
      for (int q = 0; q < norb; ++q) row[q] += mab[o[j] * norb + q];
      for (int k = j; k < n_alpha; ++k) c += maa[o[j] * norb + o[k]];
    }
    alpha_c[a] = c;
  }
#pragma omp parallel for schedule(static)
  for (long a = 0; a < dim_a; ++a) {
    const double* cm = cmap + a * norb;
    const zd* src = vec + a * dim_b;
    zd* dst = out + a * dim_b;
    for (long b = 0; b < dim_b; ++b) {
      double c = alpha_c[a] + beta_c[b];
      const long* o = occ_b + b * n_beta;
      for (int j = 0; j < n_beta; ++j) c += cm[o[j]];
      dst[b] += c * src[b];
    }
  }
  free(beta_c);
  free(alpha_c);
  free(cmap);
}

void ref_contract_nos_rows(const zd* vec, zd* out, long n_rows, long row_len, long row_stride,
                           long elem_stride, const double* coeffs, const long* occ, int nocc) {
#pragma omp parallel for schedule(static)
  for (long r = 0; r < n_rows; ++r) {
    double c = 0.0;
    for (int j = 0; j < nocc; ++j) c += coeffs[occ[r * nocc + j]];
    const zd* s = vec + r * row_stride;
    zd* d = out + r * row_stride;
    for (long q = 0; q < row_len; ++q) d[q * elem_stride] += c * s[q * elem_stride];
  }
}
