// ORACLE — test infrastructure only. A C restatement of the `la` crate's QR
// decomposition (xasmx/rust-la 0.2.0, src/decomp/qr.rs:26-238), in the
// reference's loop order with no contraction of a*b+c (the Makefile passes
// -ffp-contract=off), so its bits are the reference's on any IEEE host.
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

// QRDecomposition::new (qr.rs:26-42) with perform_householder_reflection
// (:45-105): qr (m x n) and rdiag (min(m, n)).
void oracle_qr_new(const double* a, size_t m, size_t n, double* qr, double* rdiag) {
  memcpy(qr, a, m * n * sizeof(double));
  const size_t dc = m < n ? m : n;
  for (size_t minor = 0; minor < dc; minor++) {
    double x_norm_sqr = 0.0;
    for (size_t i = minor; i < m; i++) {
      const double c = qr[i * n + minor];
      x_norm_sqr = x_norm_sqr + c * c;  // :49-53
    }
    const double a0 = qr[minor * n + minor] > 0.0 ? -sqrt(x_norm_sqr) : sqrt(x_norm_sqr);  // :58
    rdiag[minor] = a0;
    if (a0 != 0.0) {  // :62
      qr[minor * n + minor] = qr[minor * n + minor] - a0;  // :76
      for (size_t column = minor + 1; column < n; column++) {  // :92-103
        double x_dot_u = 0.0;
        for (size_t row = minor; row < m; row++)
          x_dot_u = x_dot_u + qr[row * n + minor] * qr[row * n + column];
        const double factor = x_dot_u / (a0 * qr[minor * n + minor]);
        for (size_t row = minor; row < m; row++)
          qr[row * n + column] = qr[row * n + column] + factor * qr[row * n + minor];
      }
    }
  }
}

// is_full_rank (qr.rs:108-115): 1, 0, or -1 where the reference indexes rdiag
// past its end (n > m with no zero among the first m entries).
int oracle_qr_is_full_rank(const double* rdiag, size_t m, size_t n) {
  const size_t dc = m < n ? m : n;
  for (size_t j = 0; j < n; j++) {
    if (j >= dc) return -1;
    if (rdiag[j] == 0.0) return 0;
  }
  return 1;
}

// get_h (qr.rs:119-132) and get_r (:135-148), both m x n.
void oracle_qr_get_h(const double* qr, size_t m, size_t n, double* h) {
  for (size_t i = 0; i < m; i++)
    for (size_t j = 0; j < n; j++) h[i * n + j] = i >= j ? qr[i * n + j] : 0.0;
}

void oracle_qr_get_r(const double* qr, const double* rdiag, size_t m, size_t n, double* r) {
  for (size_t i = 0; i < m; i++)
    for (size_t j = 0; j < n; j++)
      r[i * n + j] = i < j ? qr[i * n + j] : (i == j ? rdiag[i] : 0.0);
}

// get_q (qr.rs:151-194): m x m.
void oracle_qr_get_q(const double* qr, const double* rdiag, size_t m, size_t n, double* q) {
  memset(q, 0, m * m * sizeof(double));
  const size_t dc = m < n ? m : n;
  for (size_t minor = 0; minor < dc; minor++) q[minor * m + minor] = 1.0;
  for (size_t mm = dc; mm-- > 0;) {
    if (qr[mm * n + mm] != 0.0) {
      for (size_t column = mm; column < m; column++) {
        double x_dot_u = 0.0;
        for (size_t row = mm; row < m; row++)
          x_dot_u = x_dot_u + qr[row * n + mm] * q[row * m + column];
        const double factor = x_dot_u / (rdiag[mm] * qr[mm * n + mm]);
        for (size_t row = mm; row < m; row++)
          q[row * m + column] = q[row * m + column] + factor * qr[row * n + mm];
      }
    }
  }
}

// solve (qr.rs:199-238): 0 with x (n x nx), 1 for None (not full rank), 2 where
// the reference panics (b rows != m :200, is_full_rank out of bounds, an index
// past qr for n > m, or Matrix::new(n, nx, <m * nx values>) for m != n :237).
int oracle_qr_solve(const double* qr, const double* rdiag, size_t m, size_t n, const double* b,
                    size_t brows, size_t nx, double* x) {
  if (brows != m) return 2;
  const int fr = oracle_qr_is_full_rank(rdiag, m, n);
  if (fr < 0) return 2;
  if (fr == 0) return 1;
  if (m != n) return 2;  // n < m here: Matrix::new's length assert (:237)
  double* xd = (double*)malloc(m * nx * sizeof(double));
  memcpy(xd, b, m * nx * sizeof(double));
  for (size_t k = 0; k < n; k++)  // Y = Q' B (:211-223)
    for (size_t j = 0; j < nx; j++) {
      double s = 0.0;
      for (size_t i = k; i < m; i++) s = s + qr[i * n + k] * xd[i * nx + j];
      s = -s / qr[k * n + k];
      for (size_t i = k; i < m; i++) xd[i * nx + j] = xd[i * nx + j] + s * qr[i * n + k];
    }
  for (size_t k = n; k-- > 0;) {  // R X = Y (:225-235)
    for (size_t j = 0; j < nx; j++) xd[k * nx + j] = xd[k * nx + j] / rdiag[k];
    for (size_t i = 0; i < k; i++)
      for (size_t j = 0; j < nx; j++)
        xd[i * nx + j] = xd[i * nx + j] - xd[k * nx + j] * qr[i * n + k];
  }
  memcpy(x, xd, n * nx * sizeof(double));
  free(xd);
  return 0;
}
