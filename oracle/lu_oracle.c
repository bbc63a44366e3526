/*
 * ORACLE — test infrastructure only. Not part of the product and never on a
 * product code path: the tests, the smoke check and the CPU-baseline leg of the
 * benchmark call it as the checker / the timed reference CPU implementation.
 *
 * A plain-C restatement of the `la` crate's dense LU path (xasmx/rust-la 0.2.0):
 *   src/decomp/lu.rs:104-168   LUDecomposition::new  (left-looking Doolittle/Crout)
 *   src/decomp/lu.rs:170-182   is_singular / is_non_singular
 *   src/decomp/lu.rs:184-222   get_l / get_u / get_p / get_piv
 *   src/decomp/lu.rs:224-232   det
 *   src/decomp/lu.rs:237-278   solve
 *   src/matrix/mod.rs:957-980  Mul for &Matrix (naive ijk, sequential k sum)
 *   src/matrix/mmatrix.rs:82-98 mmul (same loop into a caller buffer)
 *   src/matrix/mod.rs:416-426  Matrix::id ; mod.rs:1025-1047 det/solve/inverse/is_*
 *
 * Every floating-point operation is written in the reference's order with
 * separate multiply and add (Rust never contracts a*b+c into an FMA), so this
 * file MUST be compiled with -ffp-contract=off and without fast-math. IEEE-754
 * binary64 + - * / are correctly rounded, so the results are bit-identical to
 * the Rust reference on any IEEE host.
 *
 * All matrices are row-major doubles, exactly like Matrix<f64>'s Vec<f64>.
 * The reference's `assert!` panics are returned as ORC_PANIC; its `None` as
 * ORC_NONE.
 */
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#include <math.h>

#define ORC_OK 0
#define ORC_NONE 1
#define ORC_PANIC 2

/* lu.rs:104-168. `lu` receives a copy of `a` (lu.rs:105) and is factored in
 * place; piv is the permutation vector (piv[i] = original row now at i),
 * lu.rs:108-111 and :147-149; *pospivsign flips per swap (lu.rs:151).
 * j_end (<= n) stops after column j_end-1 so the benchmark can time a bounded
 * prefix of the same factorization; pass n for the full factorization. */
void oracle_lu_factor_partial(const double* a, size_t m, size_t n, size_t j_end,
                              double* lu, uint64_t* piv, int* pospivsign) {
  memcpy(lu, a, m * n * sizeof(double));
  for (size_t i = 0; i < m; i++) piv[i] = i;
  int pos = 1;
  for (size_t j = 0; j < j_end; j++) {
    /* lu.rs:122-129: lu[i][j] = lu[i][j] - sum_{k < min(i,j)} lu[i][k]*lu[k][j] */
    for (size_t i = 0; i < m; i++) {
      double s = 0.0;
      size_t kmax = i < j ? i : j;
      for (size_t k = 0; k < kmax; k++) s = s + lu[i * n + k] * lu[k * n + j];
      lu[i * n + j] = lu[i * n + j] - s;
    }
    /* lu.rs:132-137: first row of maximum |lu[i][j]|, strict '>' */
    size_t p = j;
    for (size_t i = j + 1; i < m; i++)
      if (fabs(lu[i * n + j]) > fabs(lu[p * n + j])) p = i;
    /* lu.rs:140-152: swap entire rows, swap piv entries, flip the sign */
    if (p != j) {
      for (size_t k = 0; k < n; k++) {
        double t = lu[p * n + k];
        lu[p * n + k] = lu[j * n + k];
        lu[j * n + k] = t;
      }
      uint64_t t = piv[p]; piv[p] = piv[j]; piv[j] = t;
      pos = !pos;
    }
    /* lu.rs:156-160: divide the sub-diagonal part of column j by the pivot */
    if (j < m && lu[j * n + j] != 0.0)
      for (size_t i = j + 1; i < m; i++) lu[i * n + j] = lu[i * n + j] / lu[j * n + j];
  }
  *pospivsign = pos;
}

void oracle_lu_factor(const double* a, size_t m, size_t n,
                      double* lu, uint64_t* piv, int* pospivsign) {
  oracle_lu_factor_partial(a, m, n, n, lu, piv, pospivsign);
}

/* lu.rs:174-182. Returns 1 (non-singular), 0 (singular) or ORC_PANIC when the
 * reference's index j*n+j runs past the m*n data before a zero is found (m < n). */
int oracle_lu_is_non_singular(const double* lu, size_t m, size_t n) {
  for (size_t j = 0; j < n; j++) {
    size_t idx = j * n + j;
    if (idx >= m * n) return -ORC_PANIC;
    if (lu[idx] == 0.0) return 0;
  }
  return 1;
}

/* lu.rs:224-232: asserts square, then (+-1) * prod_{j ascending} u_jj */
int oracle_lu_det(const double* lu, size_t m, size_t n, int pospivsign, double* det) {
  if (m != n) return ORC_PANIC;
  double d = pospivsign ? 1.0 : -1.0;
  for (size_t j = 0; j < n; j++) d = d * lu[j * n + j];
  *det = d;
  return ORC_OK;
}

/* lu.rs:237-278. b is brows x nx; x is m x nx. */
int oracle_lu_solve(const double* lu, size_t m, size_t n, const uint64_t* piv,
                    const double* b, size_t brows, size_t nx, double* x) {
  if (brows != m) return ORC_PANIC;                       /* lu.rs:240 */
  int ns = oracle_lu_is_non_singular(lu, m, n);           /* lu.rs:241 */
  if (ns < 0) return ORC_PANIC;
  if (!ns) return ORC_NONE;
  size_t dest = 0;                                        /* lu.rs:245-254 */
  for (size_t i = 0; i < m; i++)
    for (size_t j = 0; j < nx; j++) x[dest++] = b[piv[i] * nx + j];
  for (size_t k = 0; k < n; k++)                          /* lu.rs:257-263 */
    for (size_t i = k + 1; i < n; i++)
      for (size_t j = 0; j < nx; j++)
        x[i * nx + j] = x[i * nx + j] - x[k * nx + j] * lu[i * n + k];
  for (size_t kk = n; kk-- > 0;) {                        /* lu.rs:266-275 */
    for (size_t j = 0; j < nx; j++) x[kk * nx + j] = x[kk * nx + j] / lu[kk * n + kk];
    for (size_t i = 0; i < kk; i++)
      for (size_t j = 0; j < nx; j++)
        x[i * nx + j] = x[i * nx + j] - x[kk * nx + j] * lu[i * n + kk];
  }
  return ORC_OK;
}

/* lu.rs:184-202: L is m x min(m,n) */
void oracle_lu_get_l(const double* lu, size_t m, size_t n, double* l) {
  size_t c = m >= n ? n : m;
  for (size_t i = 0; i < m; i++)
    for (size_t j = 0; j < c; j++)
      l[i * c + j] = i > j ? lu[i * n + j] : (i == j ? 1.0 : 0.0);
}

/* lu.rs:204-215: U is min(m,n) x n */
void oracle_lu_get_u(const double* lu, size_t m, size_t n, double* u) {
  size_t r = m >= n ? n : m;
  for (size_t i = 0; i < r; i++)
    for (size_t j = 0; j < n; j++) u[i * n + j] = i <= j ? lu[i * n + j] : 0.0;
}

/* lu.rs:217-220 with mod.rs:416-426 (id) and permute_rows: row i of P is row piv[i] of I */
void oracle_lu_get_p(const uint64_t* piv, size_t m, double* p) {
  for (size_t i = 0; i < m; i++)
    for (size_t j = 0; j < m; j++) p[i * m + j] = (piv[i] == j) ? 1.0 : 0.0;
}

/* mod.rs:957-980 (and mmatrix.rs:82-98): c[r][c] = sum_{idx ascending} a[r][idx]*b[idx][c],
 * started from zero, add-after-multiply. Rows [r0, r1) only so a bounded sample can be timed. */
int oracle_matmul_rows(const double* a, size_t m, size_t k, const double* b, size_t brows,
                       size_t n, double* c, size_t r0, size_t r1) {
  if (k != brows) return ORC_PANIC;                       /* mod.rs:961 */
  for (size_t r = r0; r < r1 && r < m; r++)
    for (size_t cc = 0; cc < n; cc++) {
      double res = 0.0;
      for (size_t idx = 0; idx < k; idx++) res = res + a[r * k + idx] * b[idx * n + cc];
      c[r * n + cc] = res;
    }
  return ORC_OK;
}

int oracle_matmul(const double* a, size_t m, size_t k, const double* b, size_t brows,
                  size_t n, double* c) {
  return oracle_matmul_rows(a, m, k, b, brows, n, c, 0, m);
}

/* mod.rs:1034-1037: assert square, LU, solve against Matrix::id(n, n).
 * Scratch: lu (n*n), piv (n), id (n*n). */
int oracle_inverse(const double* a, size_t m, size_t n, double* out,
                   double* lu, uint64_t* piv, double* id) {
  if (m != n) return ORC_PANIC;
  int pos;
  oracle_lu_factor(a, n, n, lu, piv, &pos);
  for (size_t i = 0; i < n * n; i++) id[i] = 0.0;
  for (size_t i = 0; i < n; i++) id[i * n + i] = 1.0;
  return oracle_lu_solve(lu, n, n, piv, id, n, n, out);
}

/* Normwise backward error (Rigal-Gaches), eta = ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf),
 * taken per right-hand-side column and maximised. Not part of the reference; the residual
 * sums use a two-sum/two-product compensated form so the check itself adds no error of note. */
static inline void two_sum(double a, double b, double* s, double* e) {
  double x = a + b; double bv = x - a; double av = x - bv;
  *s = x; *e = (a - av) + (b - bv);
}
static inline void two_prod(double a, double b, double* p, double* e) {
  double x = a * b; *p = x; *e = fma(a, b, -x);
}
double oracle_backward_error(const double* a, size_t n, const double* x, const double* b, size_t nrhs) {
  double anorm = 0.0;
  for (size_t i = 0; i < n; i++) {
    double s = 0.0;
    for (size_t k = 0; k < n; k++) s += fabs(a[i * n + k]);
    if (s > anorm) anorm = s;
  }
  double worst = 0.0;
  for (size_t j = 0; j < nrhs; j++) {
    double rmax = 0.0, xmax = 0.0, bmax = 0.0;
    for (size_t i = 0; i < n; i++) {
      double s = b[i * nrhs + j], c = 0.0;
      for (size_t k = 0; k < n; k++) {
        double p, pe, t, te;
        two_prod(-a[i * n + k], x[k * nrhs + j], &p, &pe);
        two_sum(s, p, &t, &te);
        s = t; c += pe + te;
      }
      double r = fabs(s + c);
      if (r > rmax) rmax = r;
      if (fabs(x[i * nrhs + j]) > xmax) xmax = fabs(x[i * nrhs + j]);
      if (fabs(b[i * nrhs + j]) > bmax) bmax = fabs(b[i * nrhs + j]);
    }
    double den = anorm * xmax + bmax;
    double eta = den > 0.0 ? rmax / den : (rmax > 0.0 ? INFINITY : 0.0);
    if (eta > worst || eta != eta) worst = eta;
  }
  return worst;
}
