// ORACLE — test infrastructure only. A C restatement of the `la` crate's
// Cholesky decomposition (xasmx/rust-la 0.2.0, src/decomp/cholesky.rs:56-145),
// in the reference's loop order and with no contraction of a*b+c (the
// Makefile passes -ffp-contract=off), so its bits are the reference's on any
// IEEE host. Used by the tests and the benchmark's CPU-baseline leg.
#include <math.h>
#include <stddef.h>
#include <string.h>

// CholeskyDecomposition::new (cholesky.rs:56-111). Rows [0, j_end) of L are
// computed into l (n x n, row-major); returns 0 (Some), or 1 (None) for a
// non-square, non-symmetric or not positive definite matrix, at the first row
// where the reference returns None.
int oracle_chol_new_partial(const double* a, size_t m, size_t n, size_t j_end, double* l) {
  if (m != n) return 1;  // cholesky.rs:57-59
  if (j_end > n) j_end = n;
  for (size_t j = 0; j < j_end; j++) {
    double d = 0.0;  // :68
    for (size_t k = 0; k < j; k++) {
      double s = 0.0;  // :76
      for (size_t i = 0; i < k; i++) s = s + l[k * n + i] * l[j * n + i];  // :77-79
      s = (a[j * n + k] - s) / l[k * n + k];  // :82
      l[j * n + k] = s;                         // :83
      d = d + s * s;                            // :86
      if (a[k * n + j] != a[j * n + k]) return 1;  // :89-91
    }
    d = a[j * n + j] - d;  // :96
    if (d <= 0.0) return 1;  // :97-100
    l[j * n + j] = sqrt(d);  // :101
    for (size_t k = j + 1; k < n; k++) l[j * n + k] = 0.0;  // :104-106
  }
  return 0;
}

int oracle_chol_new(const double* a, size_t m, size_t n, double* l) {
  return oracle_chol_new_partial(a, m, n, n, l);
}

// CholeskyDecomposition::solve (cholesky.rs:116-145): 2 (the reference's
// assert! panic) when b has a different number of rows.
int oracle_chol_solve(const double* l, size_t n, const double* b, size_t brows, size_t nx,
                      double* x) {
  if (brows != n) return 2;  // :118
  memcpy(x, b, n * nx * sizeof(double));
  // L * Y = B (:123-131)
  for (size_t k = 0; k < n; k++)
    for (size_t j = 0; j < nx; j++) {
      for (size_t i = 0; i < k; i++) x[k * nx + j] = x[k * nx + j] - x[i * nx + j] * l[k * n + i];
      x[k * nx + j] = x[k * nx + j] / l[k * n + k];
    }
  // L' * X = Y (:133-141)
  for (size_t kk = n; kk-- > 0;)
    for (size_t j = 0; j < nx; j++) {
      for (size_t i = kk + 1; i < n; i++)
        x[kk * nx + j] = x[kk * nx + j] - x[i * nx + j] * l[i * n + kk];
      x[kk * nx + j] = x[kk * nx + j] / l[kk * n + kk];
    }
  return 0;
}
