// SVD::direct (src/decomp/svd.rs:454-497) over the library's GPU Mul and LU
// inverse, with the symmetric eigendecomposition on the host.
//
//   A'A            la_matrix_mul (GPU; the reference's summation order in EXACT)
//   V, d           EigenDecomposition::new's symmetric branch (eigen.rs:755-790):
//                  Householder tridiagonalisation (tred2, eigen.rs:33-139) and
//                  the implicit QL iteration (tql2, eigen.rs:141-247), on the
//                  host in the reference's operation order; the reference
//                  keeps this step on the CPU as well
//   S, S^-1        block_diag(sqrt(d)) and la_matrix_inverse (GPU LU, lu.rs)
//   U = A V S^-1   two la_matrix_mul calls (GPU)
// For rows < cols the SVD of A' is taken and U and V swap (svd.rs:458-466).
//
// EXACT arithmetic gives the reference's bits: every GPU step has an EXACT form
// and the host steps use separate multiplies and adds (this file is compiled
// with -ffp-contract=off). The QL iteration of the reference has no iteration
// limit and never ends on non-finite data; here each eigenvalue gets at most
// 64 n + 64 sweeps and the call reports LA_UNSUPPORTED after that.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/la_gpu.h"

namespace {

// internalutil.rs:17-27: sqrt(a^2 + b^2) by the larger magnitude.
double scaled_hypot(double a, double b) {
  if (std::fabs(a) > std::fabs(b)) {
    const double r = b / a;
    return std::fabs(a) * std::sqrt(1.0 + r * r);
  }
  if (b != 0.0) {
    const double r = a / b;
    return std::fabs(b) * std::sqrt(1.0 + r * r);
  }
  return 0.0;
}

// Reduces the symmetric matrix in v (n x n, row-major) to tridiagonal form:
// d the diagonal, e the subdiagonal (e[i] couples i-1 and i), v the
// accumulated orthogonal transformation.
void tridiagonalize(size_t n, std::vector<double>& d, std::vector<double>& v,
                    std::vector<double>& e) {
  for (size_t j = 0; j < n; j++) d[j] = v[(n - 1) * n + j];
  for (size_t i = n - 1; i >= 1; i--) {
    double scale = 0.0, h = 0.0;
    for (size_t k = 0; k < i; k++) scale = scale + std::fabs(d[k]);
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
      double g = std::sqrt(h);
      if (f > 0.0) g = -g;
      e[i] = scale * g;
      h = h - f * g;
      d[i - 1] = f - g;
      for (size_t j = 0; j < i; j++) e[j] = 0.0;
      // the similarity transformation on the remaining columns
      for (size_t j = 0; j < i; j++) {
        f = d[j];
        v[j * n + i] = f;
        g = e[j] + v[j * n + j] * f;
        const double* vj = &v[0] + j;
        for (size_t k = j + 1; k < i; k++) {
          const double vkj = vj[k * n];
          g = g + vkj * d[k];
          e[k] = e[k] + vkj * f;
        }
        e[j] = g;
      }
      f = 0.0;
      for (size_t j = 0; j < i; j++) {
        e[j] = e[j] / h;
        f = f + e[j] * d[j];
      }
      const double hh = f / (h + h);
      for (size_t j = 0; j < i; j++) e[j] = e[j] - hh * d[j];
      for (size_t j = 0; j < i; j++) {
        f = d[j];
        g = e[j];
        for (size_t k = j; k < i; k++) {
          const double o = v[k * n + j];
          v[k * n + j] = o - (f * e[k] + g * d[k]);
        }
        d[j] = v[(i - 1) * n + j];
        v[i * n + j] = 0.0;
      }
    }
    d[i] = h;
  }
  // accumulate the transformations
  for (size_t i = 0; i + 1 < n; i++) {
    v[(n - 1) * n + i] = v[i * n + i];
    v[i * n + i] = 1.0;
    const double h = d[i + 1];
    if (h != 0.0) {
      for (size_t k = 0; k <= i; k++) d[k] = v[k * n + (i + 1)] / h;
      for (size_t j = 0; j <= i; j++) {
        double g = 0.0;
        for (size_t k = 0; k <= i; k++) g = g + v[k * n + (i + 1)] * v[k * n + j];
        for (size_t k = 0; k <= i; k++) v[k * n + j] = v[k * n + j] - g * d[k];
      }
    }
    for (size_t k = 0; k <= i; k++) v[k * n + (i + 1)] = 0.0;
  }
  for (size_t j = 0; j < n; j++) {
    d[j] = v[(n - 1) * n + j];
    v[(n - 1) * n + j] = 0.0;
  }
  v[(n - 1) * n + (n - 1)] = 1.0;
  e[0] = 0.0;
}

// Diagonalises the tridiagonal (d, e) by implicit QL steps, applying the
// rotations to v; eigenvalues end up in d, sorted descending with v's columns.
// false: a QL loop did not converge within its sweep limit.
bool ql_diagonalize(size_t n, std::vector<double>& e, std::vector<double>& d,
                    std::vector<double>& v) {
  for (size_t i = 1; i < n; i++) e[i - 1] = e[i];
  e[n - 1] = 0.0;
  double f = 0.0, tst1 = 0.0;
  const double eps = std::ldexp(1.0, -52);
  for (size_t l = 0; l < n; l++) {
    tst1 = std::fmax(tst1, std::fabs(d[l]) + std::fabs(e[l]));
    size_t m = l;
    while (m < n && !(std::fabs(e[m]) <= eps * tst1)) m++;
    if (m > l) {
      size_t sweeps = 0;
      for (;;) {
        if (++sweeps > 64 * n + 64) return false;
        double g = d[l];
        double p = (d[l + 1] - g) / (2.0 * e[l]);
        double r = scaled_hypot(p, 1.0);
        if (p < 0.0) r = -r;
        d[l] = e[l] / (p + r);
        d[l + 1] = e[l] * (p + r);
        const double dl1 = d[l + 1];
        double h = g - d[l];
        for (size_t i = l + 2; i < n; i++) d[i] = d[i] - h;
        f = f + h;
        p = d[m];
        double c = 1.0, c2 = c, c3 = c;
        const double el1 = e[l + 1];
        double s = 0.0, s2 = 0.0;
        for (size_t i = m; i-- > l;) {
          c3 = c2;
          c2 = c;
          s2 = s;
          g = c * e[i];
          h = c * p;
          r = scaled_hypot(p, e[i]);
          e[i + 1] = s * r;
          s = e[i] / r;
          c = p / r;
          p = c * d[i] - s * g;
          d[i + 1] = h + s * (c * g + s * d[i]);
          double* vr = v.data();
          for (size_t k = 0; k < n; k++, vr += n) {
            h = vr[i + 1];
            vr[i + 1] = s * vr[i] + c * h;
            vr[i] = c * vr[i] - s * h;
          }
        }
        p = -s * s2 * c3 * el1 * e[l] / dl1;
        e[l] = s * p;
        d[l] = c * p;
        if (std::fabs(e[l]) <= eps * tst1) break;
      }
    }
    d[l] = d[l] + f;
    e[l] = 0.0;
  }
  // selection sort, descending, columns of v alongside
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
      for (size_t j = 0; j < n; j++) std::swap(v[j * n + i], v[j * n + k]);
    }
  }
  return true;
}

void transpose(const double* a, size_t rows, size_t cols, double* t) {
  for (size_t i = 0; i < rows; i++)
    for (size_t j = 0; j < cols; j++) t[j * rows + i] = a[i * cols + j];
}

// svd.rs:465-496 for rows >= cols: u (m x m), s (m x n), v (n x n).
la_status direct_tall(la_ctx ctx, const double* a, size_t m, size_t n, double* u, double* s,
                      double* v) {
  std::vector<double> at(n * m), ata(n * n);
  transpose(a, m, n, at.data());
  la_status st = la_matrix_mul(ctx, at.data(), n, m, a, m, n, ata.data());  // :470
  if (st != LA_OK) return st;
  // EigenDecomposition::new: the symmetric branch when A'A == (A'A)' exactly
  // (eigen.rs:761-770). A NaN makes the reference take its nonsymmetric
  // branch (Hessenberg reduction, eigen.rs:791-813), which is not built.
  for (size_t j = 0; j < n; j++)
    for (size_t i = 0; i < n; i++)
      if (!(ata[i * n + j] == ata[j * n + i])) return LA_UNSUPPORTED;
  std::vector<double> d(n), e(n), vv(ata);
  tridiagonalize(n, d, vv, e);
  if (!ql_diagonalize(n, e, d, vv)) return LA_UNSUPPORTED;
  std::memcpy(v, vv.data(), n * n * sizeof(double));
  // :474-483: S = block_diag(sqrt(d)), S^-1 by the LU inverse
  std::vector<double> sq(n * n, 0.0), sinv(n * n);
  for (size_t i = 0; i < n; i++) sq[i * n + i] = std::sqrt(d[i]);
  st = la_matrix_inverse(ctx, sq.data(), n, n, sinv.data());
  if (st == LA_SINGULAR) return LA_BADSHAPE;  // inverse().unwrap() on None panics
  if (st != LA_OK) return st;
  // :484-489: S (m x n) = S cb zero, S^-1 (n x m) = S^-1 cr zero
  std::memset(s, 0, m * n * sizeof(double));
  std::memcpy(s, sq.data(), n * n * sizeof(double));
  std::vector<double> sinv_aug(n * m, 0.0), av(m * n);
  for (size_t i = 0; i < n; i++) std::memcpy(&sinv_aug[i * m], &sinv[i * n], n * sizeof(double));
  st = la_matrix_mul(ctx, a, m, n, vv.data(), n, n, av.data());  // :490 a.mul(v)
  if (st != LA_OK) return st;
  return la_matrix_mul(ctx, av.data(), m, n, sinv_aug.data(), n, m, u);  // .mul(&s_inv_aug)
}

}  // namespace

extern "C" la_status la_svd_direct(la_ctx ctx, const double* a, size_t m, size_t n, double* u,
                                   double* s, double* v) {
  if (!ctx || !a || !u || !s || !v) return LA_INVALID;
  if (m == 0 || n == 0) return LA_BADSHAPE;  // Matrix::new asserts
  if (m >= n) return direct_tall(ctx, a, m, n, u, s, v);
  // svd.rs:458-466: the SVD of A' (n x m), U and V swapped, S transposed
  std::vector<double> at(n * m), st_(n * m);
  transpose(a, m, n, at.data());
  la_status r = direct_tall(ctx, at.data(), n, m, v, st_.data(), u);
  if (r == LA_OK) transpose(st_.data(), n, m, s);
  return r;
}
