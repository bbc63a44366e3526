/*
 * ORACLE — test infrastructure only. Not part of the product and never on a
 * product code path: the tests call it as the checker.
 *
 * A plain-C restatement of the `la` crate's SVD::direct (xasmx/rust-la 0.2.0)
 * and of the pieces it calls:
 *   src/decomp/svd.rs:454-497     SVD::direct (A'A, its eigenvectors V, the
 *                                 singular values sqrt(d), U = A V S^-1)
 *   src/decomp/eigen.rs:755-790   EigenDecomposition::new, symmetric branch
 *   src/decomp/eigen.rs:33-139    tred2 (Householder tridiagonalisation)
 *   src/decomp/eigen.rs:141-247   tql2 (implicit QL, eigenvalues sorted descending)
 *   src/internalutil.rs:17-27     hypot (JAMA's scaled form)
 *   src/matrix/mod.rs:428-466, 579-664   zero, block_diag, cr, cb, t
 * Mul and inverse are the LU oracle's (lu_oracle.c: mod.rs:957-980, 1034-1037).
 *
 * Every floating-point operation follows the reference's order with separate
 * multiplies and adds: compile with -ffp-contract=off and without fast-math.
 *
 * Two departures, where the reference cannot return:
 *  - A'A with a NaN is not symmetric under `==`, and the reference then takes
 *    its nonsymmetric branch (orthes / hqr2, eigen.rs:249-750), which is not
 *    restated here: ORC_UNSUPPORTED.
 *  - tql2 has no iteration limit; on non-finite data its QL loop never ends.
 *    Here a limit of 64 * n sweeps per eigenvalue ends it: ORC_NOT_FINITE.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_NONE 1
#define ORC_PANIC 2
#define ORC_UNSUPPORTED 3
#define ORC_NOT_FINITE 4

int oracle_matmul(const double* a, size_t m, size_t k, const double* b, size_t brows,
                  size_t n, double* c);
int oracle_inverse(const double* a, size_t m, size_t n, double* out, double* lu, uint64_t* piv,
                   double* id);

/* internalutil.rs:17-27 */
static double hypot_ref(double a, double b) {
  if (fabs(a) > fabs(b)) {
    double r = b / a;
    return fabs(a) * sqrt(1.0 + r * r);
  } else if (b != 0.0) {
    double r = a / b;
    return fabs(b) * sqrt(1.0 + r * r);
  }
  return 0.0;
}

/* mod.rs:653-664: the transpose (rows x cols -> cols x rows). */
static void transpose(const double* a, size_t rows, size_t cols, double* t) {
  for (size_t i = 0; i < rows; i++)
    for (size_t j = 0; j < cols; j++) t[j * rows + i] = a[i * cols + j];
}

/* eigen.rs:33-139 (v: n x n row-major, holds A on entry). */
static void tred2(size_t n, double* d, double* v, double* e) {
  for (size_t j = 0; j < n; j++) d[j] = v[(n - 1) * n + j];
  for (size_t i = n - 1; i >= 1; i--) {
    double scale = 0.0, h = 0.0;
    for (size_t k = 0; k < i; k++) scale = scale + fabs(d[k]);
    if (scale == 0.0) {
      e[i] = d[i - 1];
      for (size_t j = 0; j < i; j++) {
        d[j] = v[(i - 1) * n + j];
        v[i * n + j] = 0.0;
        v[j * n + i] = 0.0;
      }
    } else {
      for (size_t k = 0; k < i; k++) {
        d[k] = d[k] / scale;
        h = h + d[k] * d[k];
      }
      double f = d[i - 1];
      double g = sqrt(h);
      if (f > 0.0) g = -g;
      e[i] = scale * g;
      h = h - f * g;
      d[i - 1] = f - g;
      for (size_t j = 0; j < i; j++) e[j] = 0.0;
      for (size_t j = 0; j < i; j++) {
        f = d[j];
        v[j * n + i] = f;
        g = e[j] + v[j * n + j] * f;
        for (size_t k = j + 1; k < i; k++) {
          g = g + v[k * n + j] * d[k];
          e[k] = e[k] + v[k * n + j] * f;
        }
        e[j] = g;
      }
      f = 0.0;
      for (size_t j = 0; j < i; j++) {
        e[j] = e[j] / h;
        f = f + e[j] * d[j];
      }
      double hh = f / (h + h);
      for (size_t j = 0; j < i; j++) e[j] = e[j] - hh * d[j];
      for (size_t j = 0; j < i; j++) {
        f = d[j];
        g = e[j];
        for (size_t k = j; k < i; k++) {
          double orig = v[k * n + j];
          v[k * n + j] = orig - (f * e[k] + g * d[k]);
        }
        d[j] = v[(i - 1) * n + j];
        v[i * n + j] = 0.0;
      }
    }
    d[i] = h;
  }
  for (size_t i = 0; i + 1 < n; i++) {
    double orig = v[i * n + i];
    v[(n - 1) * n + i] = orig;
    v[i * n + i] = 1.0;
    double h = d[i + 1];
    if (h != 0.0) {
      for (size_t k = 0; k < i + 1; k++) d[k] = v[k * n + (i + 1)] / h;
      for (size_t j = 0; j < i + 1; j++) {
        double g = 0.0;
        for (size_t k = 0; k < i + 1; k++) g = g + v[k * n + (i + 1)] * v[k * n + j];
        for (size_t k = 0; k < i + 1; k++) {
          double o = v[k * n + j];
          v[k * n + j] = o - g * d[k];
        }
      }
    }
    for (size_t k = 0; k < i + 1; k++) v[k * n + (i + 1)] = 0.0;
  }
  for (size_t j = 0; j < n; j++) {
    d[j] = v[(n - 1) * n + j];
    v[(n - 1) * n + j] = 0.0;
  }
  v[(n - 1) * n + (n - 1)] = 1.0;
  e[0] = 0.0;
}

/* eigen.rs:141-247. Returns ORC_NOT_FINITE when a QL loop does not converge
 * within its limit (the reference would loop forever). */
static int tql2(size_t n, double* e, double* d, double* v) {
  for (size_t i = 1; i < n; i++) e[i - 1] = e[i];
  e[n - 1] = 0.0;
  double f = 0.0, tst1 = 0.0;
  const double eps = ldexp(1.0, -52);
  for (size_t l = 0; l < n; l++) {
    tst1 = fmax(tst1, fabs(d[l]) + fabs(e[l]));
    size_t m = l;
    while (m < n) {
      if (fabs(e[m]) <= eps * tst1) break;
      m++;
    }
    if (m > l) {
      size_t sweeps = 0;
      for (;;) {
        if (++sweeps > 64 * n + 64) return ORC_NOT_FINITE;
        double g = d[l];
        double p = (d[l + 1] - g) / (2.0 * e[l]);
        double r = hypot_ref(p, 1.0);
        if (p < 0.0) r = -r;
        d[l] = e[l] / (p + r);
        d[l + 1] = e[l] * (p + r);
        double dl1 = d[l + 1];
        double h = g - d[l];
        for (size_t i = l + 2; i < n; i++) d[i] = d[i] - h;
        f = f + h;
        p = d[m];
        double c = 1.0, c2 = c, c3 = c;
        double el1 = e[l + 1];
        double s = 0.0, s2 = 0.0;
        for (size_t i = m; i-- > l;) {
          c3 = c2;
          c2 = c;
          s2 = s;
          g = c * e[i];
          h = c * p;
          r = hypot_ref(p, e[i]);
          e[i + 1] = s * r;
          s = e[i] / r;
          c = p / r;
          p = c * d[i] - s * g;
          d[i + 1] = h + s * (c * g + s * d[i]);
          for (size_t k = 0; k < n; k++) {
            h = v[k * n + (i + 1)];
            v[k * n + (i + 1)] = s * v[k * n + i] + c * h;
            v[k * n + i] = c * v[k * n + i] - s * h;
          }
        }
        p = -s * s2 * c3 * el1 * e[l] / dl1;
        e[l] = s * p;
        d[l] = c * p;
        if (fabs(e[l]) <= eps * tst1) break;
      }
    }
    d[l] = d[l] + f;
    e[l] = 0.0;
  }
  for (size_t i = 0; i + 1 < n; i++) {
    size_t k = i;
    double p = d[i];
    for (size_t j = i + 1; j < n; j++)
      if (d[j] > p) {
        k = j;
        p = d[j];
      }
    if (k != i) {
      d[k] = d[i];
      d[i] = p;
      for (size_t j = 0; j < n; j++) {
        p = v[j * n + i];
        v[j * n + i] = v[j * n + k];
        v[j * n + k] = p;
      }
    }
  }
  return ORC_OK;
}

/* eigen.rs:755-790, symmetric branch: d (n) the real eigenvalues (descending),
 * e (n) the imaginary parts (zeros), v (n x n) the eigenvectors as columns. */
int oracle_eig_sym(const double* a, size_t n, double* d, double* e, double* v) {
  for (size_t j = 0; j < n; j++)
    for (size_t i = 0; i < n; i++)
      if (!(a[i * n + j] == a[j * n + i])) return ORC_UNSUPPORTED;
  memcpy(v, a, n * n * sizeof(double));
  tred2(n, d, v, e);
  return tql2(n, e, d, v);
}

/* svd.rs:465-496 for rows >= cols: u (m x m), s (m x n), v (n x n). */
static int direct_tall(const double* a, size_t m, size_t n, double* u, double* s, double* v) {
  int st = ORC_OK;
  double* at = malloc(n * m * sizeof(double));
  double* ata = malloc(n * n * sizeof(double));
  double* d = malloc(n * sizeof(double));
  double* e = malloc(n * sizeof(double));
  double* sq = calloc(n * n, sizeof(double));
  double* sinv = malloc(n * n * sizeof(double));
  double* lu = malloc(n * n * sizeof(double));
  uint64_t* piv = malloc(n * sizeof(uint64_t));
  double* id = malloc(n * n * sizeof(double));
  double* sinv_aug = calloc(n * m, sizeof(double));
  double* av = malloc(m * n * sizeof(double));
  if (!at || !ata || !d || !e || !sq || !sinv || !lu || !piv || !id || !sinv_aug || !av) {
    st = ORC_UNSUPPORTED;
    goto out;
  }
  transpose(a, m, n, at);
  oracle_matmul(at, n, m, a, m, n, ata); /* :470 */
  st = oracle_eig_sym(ata, n, d, e, v);   /* :471-473 */
  if (st != ORC_OK) goto out;
  for (size_t i = 0; i < n; i++) sq[i * n + i] = sqrt(d[i]); /* :474, :482 block_diag */
  st = oracle_inverse(sq, n, n, sinv, lu, piv, id);        /* :483 */
  if (st == ORC_NONE) {
    st = ORC_PANIC; /* inverse().unwrap() on None */
    goto out;
  }
  /* :484-489: S (m x n) = S cb zero; S^-1 (n x m) = S^-1 cr zero */
  memset(s, 0, m * n * sizeof(double));
  memcpy(s, sq, n * n * sizeof(double));
  for (size_t i = 0; i < n; i++) memcpy(sinv_aug + i * m, sinv + i * n, n * sizeof(double));
  oracle_matmul(a, m, n, v, n, n, av);          /* :490 a.mul(v) */
  oracle_matmul(av, m, n, sinv_aug, n, m, u);   /*      .mul(&s_inv_aug) */
out:
  free(at); free(ata); free(d); free(e); free(sq); free(sinv); free(lu); free(piv); free(id);
  free(sinv_aug); free(av);
  return st;
}

/* svd.rs:454-497: u (m x m), s (m x n), v (n x n) with A = U S V' where
 * the reference's arithmetic holds. ORC_PANIC where inverse().unwrap() panics
 * (a zero singular value). */
int oracle_svd_direct(const double* a, size_t m, size_t n, double* u, double* s, double* v) {
  if (m >= n) return direct_tall(a, m, n, u, s, v);
  /* :458-466: the SVD of a' (n x m) with u and v swapped and s transposed */
  double* at = malloc(n * m * sizeof(double));
  double* st_ = malloc(n * m * sizeof(double));
  if (!at || !st_) {
    free(at);
    free(st_);
    return ORC_UNSUPPORTED;
  }
  transpose(a, m, n, at);
  int r = direct_tall(at, n, m, v, st_, u); /* u' (n x n) -> v, v' (m x m) -> u */
  if (r == ORC_OK) transpose(st_, n, m, s);
  free(at);
  free(st_);
  return r;
}
