/*
 * ORACLE — test infrastructure only (the timed reference-CPU leg of the
 * benchmark). Multi-threaded form of the restatement in lu_oracle.c:
 * the same left-looking loop of src/decomp/lu.rs:116-161, with the rows at or
 * below the diagonal of the column update (lu.rs:122-129) split across OpenMP
 * threads. Each row's dot product is still summed by one thread in ascending k,
 * and the rows above the diagonal keep their order, so the result is
 * bit-identical to lu_oracle.c and to the single-threaded reference; only the
 * wall time changes. Compile with -ffp-contract=off -fopenmp.
 */
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#include <math.h>
#include <omp.h>

int oracle_mt_max_threads(void) { return omp_get_max_threads(); }

void oracle_mt_lu_factor_partial(const double* a, size_t m, size_t n, size_t j_end,
                                 double* lu, uint64_t* piv, int* pospivsign, int nthreads) {
  memcpy(lu, a, m * n * sizeof(double));
  for (size_t i = 0; i < m; i++) piv[i] = i;
  int pos = 1;
  for (size_t j = 0; j < j_end; j++) {
    /* Rows i < j read column j's new values of the rows above them
     * (lu.rs:125 with k < i), so they stay in order on one thread. */
    size_t iu = j < m ? j : m;
    for (size_t i = 0; i < iu; i++) {
      double s = 0.0;
      for (size_t k = 0; k < i; k++) s = s + lu[i * n + k] * lu[k * n + j];
      lu[i * n + j] = lu[i * n + j] - s;
    }
    /* Rows i >= j only read finished rows k < j: independent. */
    #pragma omp parallel for schedule(static) num_threads(nthreads)
    for (size_t i = iu; i < m; i++) {
      double s = 0.0;
      for (size_t k = 0; k < j; k++) s = s + lu[i * n + k] * lu[k * n + j];
      lu[i * n + j] = lu[i * n + j] - s;
    }
    size_t p = j;
    for (size_t i = j + 1; i < m; i++)
      if (fabs(lu[i * n + j]) > fabs(lu[p * n + j])) p = i;
    if (p != j) {
      for (size_t k = 0; k < n; k++) {
        double t = lu[p * n + k]; lu[p * n + k] = lu[j * n + k]; lu[j * n + k] = t;
      }
      uint64_t t = piv[p]; piv[p] = piv[j]; piv[j] = t;
      pos = !pos;
    }
    if (j < m && lu[j * n + j] != 0.0) {
      double d = lu[j * n + j];
      #pragma omp parallel for schedule(static) num_threads(nthreads)
      for (size_t i = j + 1; i < m; i++) lu[i * n + j] = lu[i * n + j] / d;
    }
  }
  *pospivsign = pos;
}

/* lu.rs:257-275 with the right-hand-side columns split across threads: each
 * column's forward/back substitution is independent and keeps its own order. */
void oracle_mt_lu_solve_nocheck(const double* lu, size_t n, const uint64_t* piv,
                                const double* b, size_t nx, double* x, int nthreads) {
  for (size_t i = 0; i < n; i++)
    for (size_t j = 0; j < nx; j++) x[i * nx + j] = b[piv[i] * nx + j];
  #pragma omp parallel for schedule(static) num_threads(nthreads)
  for (size_t j = 0; j < nx; j++) {
    for (size_t k = 0; k < n; k++)
      for (size_t i = k + 1; i < n; i++)
        x[i * nx + j] = x[i * nx + j] - x[k * nx + j] * lu[i * n + k];
    for (size_t kk = n; kk-- > 0;) {
      x[kk * nx + j] = x[kk * nx + j] / lu[kk * n + kk];
      for (size_t i = 0; i < kk; i++)
        x[i * nx + j] = x[i * nx + j] - x[kk * nx + j] * lu[i * n + kk];
    }
  }
}

/* mod.rs:957-980 with output rows split across threads (each entry's k-sum unchanged). */
void oracle_mt_matmul_rows(const double* a, size_t m, size_t k, const double* b,
                           size_t n, double* c, size_t r0, size_t r1, int nthreads) {
  if (r1 > m) r1 = m;
  #pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (size_t r = r0; r < r1; r++)
    for (size_t cc = 0; cc < n; cc++) {
      double res = 0.0;
      for (size_t idx = 0; idx < k; idx++) res = res + a[r * k + idx] * b[idx * n + cc];
      c[r * n + cc] = res;
    }
}
