// QR decomposition (QRDecomposition, src/decomp/qr.rs:26-238) and
// Matrix::pinverse (src/matrix/mod.rs:1049-1057).
//
// The reference reflects one column at a time (Householder, unblocked): for
// column `minor` it sums the squares of rows minor.. in ascending order, takes
// a = -/+ sqrt, stores a in rdiag, subtracts a from the diagonal entry, and for
// every later column forms the dot product with that Householder vector
// (ascending rows), the factor dot / (a u_k) and the update t += factor u.
// get_q applies the reflections in reverse to a matrix with ones on its first
// min(m, n) diagonal entries; solve applies them to b with the factor
// -(dot / u_k) and back-substitutes with R.
//
// EXACT: every reflection is one launch of qr_reflect_kernel, one thread per
// target column, each walking the rows in the reference's order with unfused
// products and sums, so the factors, Q and the solution are bit-identical to
// the reference; the column norm is one thread's ascending sum.
// FAST, from 128 columns while the rows fit one cluster: blocks of 64
// reflections in compact WY form (qr_blocked.cu), and get_q and solve block by
// block. FAST otherwise: qr_reflect_fast_kernel, 4 target columns per CTA and
// 64 row slots (many CTAs per SM, short dependent chains), the dot products
// reduced by warp shuffles and across warps, then the update with FMA; in the
// factorization the CTA that holds the next column also takes that column's
// norm and diagonal once its update is done, so each column costs one launch.
// The back-substitution of solve is the wavefront upper solve on R (the
// reference's descending term order, then the division by rdiag).
#include <cstring>

#include "la_internal.cuh"

struct la_qr_handle {
  la_ctx ctx = nullptr;
  size_t m = 0, n = 0, ld = 0;
  double* d_qr = nullptr;     // m x n, pitch ld: R above the diagonal, Householder vectors below
  double* d_rdiag = nullptr;  // min(m, n)
  std::vector<double> rdiag;  // host copy (is_full_rank)
  int arith = LA_ARITH_FAST;
  double* d_gram = nullptr;   // blocked FAST factorization: V'V of each block (else null)
};

namespace {

size_t pad4q(size_t x) { return (x + 3) & ~size_t(3); }

struct QBuf {
  la_ctx ctx;
  void* p = nullptr;
  explicit QBuf(la_ctx c) : ctx(c) {}
  ~QBuf() { la_device_free(ctx, p); }
  la_status alloc(size_t bytes) { return la_device_alloc(ctx, &p, bytes); }
  double* d() { return static_cast<double*>(p); }
};

// Column `minor`: the sum of squares of rows [minor, m) (qr.rs:49-53), a
// (:58), rdiag[minor] = a, and the diagonal entry minus a (:76). One warp.
template <bool EXACT>
__global__ void qr_norm_kernel(double* Q, size_t ld, int m, int minor, double* rdiag) {
  const int lane = threadIdx.x;
  double x = 0.0;
  if (EXACT) {
    if (lane == 0)
      for (int i = minor; i < m; i++) {
        const double c = Q[(size_t)i * ld + minor];
        x = __dadd_rn(x, __dmul_rn(c, c));
      }
  } else {
    for (int i = minor + lane; i < m; i += 32) {
      const double c = Q[(size_t)i * ld + minor];
      x = fma(c, c, x);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
  }
  if (lane == 0) {
    const double q = Q[(size_t)minor * ld + minor];
    const double a = q > 0.0 ? -sqrt(x) : sqrt(x);
    rdiag[minor] = a;
    if (a != 0.0) Q[(size_t)minor * ld + minor] = q - a;
  }
}

// The reflection by column `ucol` of U (rows [r0, m)) applied to columns
// [c0, c1) of T, one thread per column:
//   dot = sum over rows of u * t (ascending), factor = dot / den,
//   t = t + factor * u.
// mode 0 (factorization, qr.rs:92-103): skipped when a = rdiag[ucol] is 0,
//   den = a * u_r0;
// mode 1 (get_q, :167-189): skipped when u_r0 is 0, den = rdiag[ucol] * u_r0;
// mode 2 (solve, :212-222): den = -u_r0 (dot / -u equals -(dot / u) exactly).
// U and T may be the same matrix (mode 0): the columns differ.
template <bool EXACT>
__global__ void qr_reflect_kernel(const double* U, size_t ldu, int ucol, int r0, int m,
                                  const double* rdiag, double* T, size_t ldt, int c0, int c1,
                                  int mode) {
  const int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  const double u0 = U[(size_t)r0 * ldu + ucol];
  double den;
  if (mode == 0) {
    const double a = rdiag[ucol];
    if (a == 0.0) return;
    den = EXACT ? __dmul_rn(a, u0) : a * u0;
  } else if (mode == 1) {
    if (u0 == 0.0) return;
    den = EXACT ? __dmul_rn(rdiag[ucol], u0) : rdiag[ucol] * u0;
  } else {
    den = -u0;
  }
  if (c >= c1) return;
  double dot = 0.0;
  for (int row = r0; row < m; row++) {
    const double u = U[(size_t)row * ldu + ucol];
    const double t = T[(size_t)row * ldt + c];
    dot = EXACT ? __dadd_rn(dot, __dmul_rn(u, t)) : fma(u, t, dot);
  }
  const double factor = dot / den;
  for (int row = r0; row < m; row++) {
    const double u = U[(size_t)row * ldu + ucol];
    double* t = T + (size_t)row * ldt + c;
    *t = EXACT ? __dadd_rn(*t, __dmul_rn(factor, u)) : fma(factor, u, *t);
  }
}

// FAST form of qr_reflect_kernel (same modes and denominators): CTA b takes
// columns [c0 + 4 b, c0 + 4 b + 4) of T; thread (s, c) = (tid / 4, tid % 4)
// walks rows r0 + s, r0 + s + 64, ... of its column, four rows per step with
// their loads issued together. Narrow column tiles give many CTAs per SM and
// short dependent chains (the products are cheap, the L2 latency is not); the
// 64 partial dot products of a column are combined by shuffles within each
// warp (its 8 row slots) and then across the 8 warps. When next >= 0
// (factorization) the CTA that holds column `next` then takes its norm over
// rows [next, m), a = -/+ sqrt, rdiag[next] = a and the diagonal entry minus a
// (qr.rs:49-76 for the next step), so every column costs one launch.
constexpr int RF_C = 4, RF_R = 64;  // 256 threads
__global__ void __launch_bounds__(RF_C * RF_R)
qr_reflect_fast_kernel(const double* U, size_t ldu, int ucol, int r0, int m, double* rdiag,
                       double* T, size_t ldt, int c0, int c1, int mode, int next) {
  __shared__ double red[8][RF_C];
  __shared__ double fac[RF_C];
  __shared__ double nred[8];
  const int tid = threadIdx.x, cl = tid % RF_C, rs = tid / RF_C;
  const int lane = tid & 31, warp = tid >> 5;
  const int cb = c0 + blockIdx.x * RF_C;
  const int c = cb + cl;
  const double u0 = U[(size_t)r0 * ldu + ucol];
  double den = 1.0;
  bool skip = false;
  if (mode == 0) {
    const double a = rdiag[ucol];
    skip = a == 0.0;
    den = a * u0;
  } else if (mode == 1) {
    skip = u0 == 0.0;
    den = rdiag[ucol] * u0;
  } else {
    den = -u0;
  }
  if (!skip) {
    double dot = 0.0;
    if (c < c1) {
      int row = r0 + rs;
      for (; row + 3 * RF_R < m; row += 4 * RF_R) {
        const double ua = U[(size_t)row * ldu + ucol], ub = U[(size_t)(row + RF_R) * ldu + ucol];
        const double uc = U[(size_t)(row + 2 * RF_R) * ldu + ucol];
        const double ud = U[(size_t)(row + 3 * RF_R) * ldu + ucol];
        const double ta = T[(size_t)row * ldt + c], tb = T[(size_t)(row + RF_R) * ldt + c];
        const double tc = T[(size_t)(row + 2 * RF_R) * ldt + c];
        const double td = T[(size_t)(row + 3 * RF_R) * ldt + c];
        dot = fma(ua, ta, dot);
        dot = fma(ub, tb, dot);
        dot = fma(uc, tc, dot);
        dot = fma(ud, td, dot);
      }
      for (; row < m; row += RF_R) dot = fma(U[(size_t)row * ldu + ucol], T[(size_t)row * ldt + c], dot);
    }
    // the 8 row slots of a column within a warp (lanes cl, cl + 4, ..., cl + 28)
    dot += __shfl_xor_sync(0xffffffffu, dot, 4);
    dot += __shfl_xor_sync(0xffffffffu, dot, 8);
    dot += __shfl_xor_sync(0xffffffffu, dot, 16);
    if (lane < RF_C) red[warp][lane] = dot;
    __syncthreads();
    if (tid < RF_C) {
      double sum = 0.0;
#pragma unroll
      for (int w = 0; w < 8; w++) sum += red[w][tid];
      fac[tid] = sum / den;
    }
    __syncthreads();
    const double f = fac[cl];
    if (c < c1) {
      int row = r0 + rs;
      for (; row + 3 * RF_R < m; row += 4 * RF_R) {
        double* ta = T + (size_t)row * ldt + c;
        double* tb = T + (size_t)(row + RF_R) * ldt + c;
        double* tc = T + (size_t)(row + 2 * RF_R) * ldt + c;
        double* td = T + (size_t)(row + 3 * RF_R) * ldt + c;
        const double ua = U[(size_t)row * ldu + ucol], ub = U[(size_t)(row + RF_R) * ldu + ucol];
        const double uc = U[(size_t)(row + 2 * RF_R) * ldu + ucol];
        const double ud = U[(size_t)(row + 3 * RF_R) * ldu + ucol];
        const double va = *ta, vb = *tb, vc = *tc, vd = *td;
        *ta = fma(f, ua, va);
        *tb = fma(f, ub, vb);
        *tc = fma(f, uc, vc);
        *td = fma(f, ud, vd);
      }
      for (; row < m; row += RF_R) {
        double* t = T + (size_t)row * ldt + c;
        *t = fma(f, U[(size_t)row * ldu + ucol], *t);
      }
    }
  }
  if (next >= 0 && next >= cb && next < cb + RF_C) {
    __syncthreads();  // this CTA's updates of column `next` are visible to the block
    double x = 0.0;
    for (int row = next + tid; row < m; row += RF_C * RF_R) {
      const double v = T[(size_t)row * ldt + next];
      x = fma(v, v, x);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    if (lane == 0) nred[warp] = x;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < 8; w++) t += nred[w];
      const double q = T[(size_t)next * ldt + next];
      const double a = q > 0.0 ? -sqrt(t) : sqrt(t);
      rdiag[next] = a;
      if (a != 0.0) T[(size_t)next * ldt + next] = q - a;
    }
  }
}

// get_r (qr.rs:135-148, which = 0), get_h (:119-132, which = 1), m x n, and
// the n x n upper block of R for the back-substitution (which = 0, rows < n).
__global__ void qr_extract_kernel(const double* Q, size_t ld, const double* rdiag, int rows,
                                  int n, double* out, size_t ldo, int which) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)rows * n) return;
  const int i = (int)(idx / n), j = (int)(idx % n);
  double v;
  if (which == 0) v = i < j ? Q[(size_t)i * ld + j] : (i == j ? rdiag[i] : 0.0);
  else v = i >= j ? Q[(size_t)i * ld + j] : 0.0;
  out[(size_t)i * ldo + j] = v;
}

// The m x m start of get_q: zeros, ones on the first dc diagonal entries.
__global__ void qr_q_init_kernel(double* Qm, size_t ldq, int m, int dc) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)m * m) return;
  const int i = (int)(idx / m), j = (int)(idx % m);
  Qm[(size_t)i * ldq + j] = (i == j && i < dc) ? 1.0 : 0.0;
}

int blocks_for(size_t total, int t) { return (int)((total + t - 1) / t); }

}  // namespace

namespace {

constexpr int QT = 128;

la_status qr_check_ctx(la_ctx ctx) {
  if (!ctx) return LA_INVALID;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaSetDevice");
  return LA_OK;
}

template <bool EXACT>
la_status launch_reflect(la_ctx ctx, const double* U, size_t ldu, int ucol, int r0, int m,
                         double* rdiag, double* T, size_t ldt, int c0, int c1, int mode) {
  if (c1 <= c0) return LA_OK;
  qr_reflect_kernel<EXACT><<<blocks_for((size_t)(c1 - c0), QT), QT, 0, ctx->stream>>>(
      U, ldu, ucol, r0, m, rdiag, T, ldt, c0, c1, mode);
  ctx->launches++;
  return la_check_launch(ctx, "qr_reflect_kernel");
}

// FAST reflection; next >= 0 also prepares column `next` (factorization). At
// least one CTA runs even for an empty column range when `next` needs it.
la_status launch_reflect_fast(la_ctx ctx, const double* U, size_t ldu, int ucol, int r0, int m,
                              double* rdiag, double* T, size_t ldt, int c0, int c1, int mode,
                              int next) {
  if (c1 <= c0 && next < 0) return LA_OK;
  const int blocks = std::max(1, (c1 - c0 + RF_C - 1) / RF_C);
  qr_reflect_fast_kernel<<<blocks, RF_C * RF_R, 0, ctx->stream>>>(U, ldu, ucol, r0, m, rdiag, T,
                                                                  ldt, c0, c1, mode, next);
  ctx->launches++;
  return la_check_launch(ctx, "qr_reflect_fast_kernel");
}

la_status reflect(la_ctx ctx, bool exact, const double* U, size_t ldu, int ucol, int r0, int m,
                  double* rdiag, double* T, size_t ldt, int c0, int c1, int mode) {
  return exact ? launch_reflect<true>(ctx, U, ldu, ucol, r0, m, rdiag, T, ldt, c0, c1, mode)
               : launch_reflect_fast(ctx, U, ldu, ucol, r0, m, rdiag, T, ldt, c0, c1, mode, -1);
}

// qr.rs:26-42. EXACT: one norm launch and one reflection launch per column;
// FAST: the first column's norm, then one launch per column (the reflection
// and the next column's norm).
la_status qr_factor(la_ctx ctx, la_qr h) {
  const int m = (int)h->m, n = (int)h->n, dc = std::min(m, n);
  const bool exact = h->arith == LA_ARITH_EXACT;
  if (!exact && qr_blocked_supported(ctx, m, n)) {
    void* g = nullptr;
    const size_t nblocks = (size_t)(dc + QR_BLOCK - 1) / QR_BLOCK;
    LA_TRY(la_device_alloc(ctx, &g, nblocks * QR_BLOCK * QR_BLOCK * sizeof(double)));
    h->d_gram = static_cast<double*>(g);
    const la_status s = qr_blocked_factor(ctx, h->d_qr, h->ld, m, n, h->d_rdiag, h->d_gram);
    if (s != LA_UNSUPPORTED) {
      LA_TRY(s);
      h->rdiag.assign((size_t)dc, 0.0);
      LA_CUDA(ctx, cudaMemcpyAsync(h->rdiag.data(), h->d_rdiag, (size_t)dc * sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream));
      return la_sync_and_check(ctx, "qr factorization (blocked)");
    }
    la_device_free(ctx, h->d_gram);
    h->d_gram = nullptr;
  }
  if (!exact) {
    qr_norm_kernel<false><<<1, 32, 0, ctx->stream>>>(h->d_qr, h->ld, m, 0, h->d_rdiag);
    ctx->launches++;
    LA_TRY(la_check_launch(ctx, "qr_norm_kernel"));
  }
  for (int minor = 0; minor < dc; minor++) {
    if (exact) {
      qr_norm_kernel<true><<<1, 32, 0, ctx->stream>>>(h->d_qr, h->ld, m, minor, h->d_rdiag);
      ctx->launches++;
      LA_TRY(la_check_launch(ctx, "qr_norm_kernel"));
      LA_TRY(reflect(ctx, true, h->d_qr, h->ld, minor, minor, m, h->d_rdiag, h->d_qr, h->ld,
                     minor + 1, n, 0));
    } else {
      LA_TRY(launch_reflect_fast(ctx, h->d_qr, h->ld, minor, minor, m, h->d_rdiag, h->d_qr,
                                 h->ld, minor + 1, n, 0, minor + 1 < dc ? minor + 1 : -1));
    }
  }
  h->rdiag.assign((size_t)dc, 0.0);
  LA_CUDA(ctx, cudaMemcpyAsync(h->rdiag.data(), h->d_rdiag, (size_t)dc * sizeof(double),
                               cudaMemcpyDeviceToHost, ctx->stream));
  return la_sync_and_check(ctx, "qr factorization");
}

la_status qr_alloc(la_ctx ctx, size_t m, size_t n, la_qr* out) {
  if (m == 0 || n == 0) return LA_BADSHAPE;  // Matrix::new asserts (mod.rs:209)
  if (m > (size_t)INT32_MAX / 2 || n > (size_t)INT32_MAX / 2) return LA_UNSUPPORTED;
  la_qr h = new (std::nothrow) la_qr_handle();
  if (!h) return LA_NOMEM;
  h->ctx = ctx;
  h->m = m;
  h->n = n;
  h->ld = pad4q(n);
  h->arith = ctx->arith;
  void* p = nullptr;
  la_status s = la_device_alloc(ctx, &p, m * h->ld * sizeof(double));
  if (s != LA_OK) { delete h; return s; }
  h->d_qr = static_cast<double*>(p);
  s = la_device_alloc(ctx, &p, std::min(m, n) * sizeof(double));
  if (s != LA_OK) { la_qr_free(h); return s; }
  h->d_rdiag = static_cast<double*>(p);
  *out = h;
  return LA_OK;
}

la_status qr_new_common(la_ctx ctx, la_qr h, la_qr* out) {
  la_status s = qr_factor(ctx, h);
  if (s != LA_OK) {
    la_qr_free(h);
    return s;
  }
  *out = h;
  return LA_OK;
}

// is_full_rank (qr.rs:108-115): 1/0, or LA_BADSHAPE where it indexes rdiag
// past min(m, n) (n > m and no zero among the first m entries).
la_status qr_full_rank(la_qr h, int* out) {
  const size_t dc = std::min(h->m, h->n);
  for (size_t j = 0; j < h->n; j++) {
    if (j >= dc) return LA_BADSHAPE;
    if (h->rdiag[j] == 0.0) { *out = 0; return LA_OK; }
  }
  *out = 1;
  return LA_OK;
}

la_status qr_extract_host(la_qr h, int which, double* out) {
  la_ctx ctx = h->ctx;
  LA_TRY(qr_check_ctx(ctx));
  const size_t total = h->m * h->n;
  QBuf d(ctx);
  LA_TRY(d.alloc(total * sizeof(double)));
  qr_extract_kernel<<<blocks_for(total, 256), 256, 0, ctx->stream>>>(
      h->d_qr, h->ld, h->d_rdiag, (int)h->m, (int)h->n, d.d(), h->n, which);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "qr_extract_kernel"));
  LA_CUDA(ctx, cudaMemcpyAsync(out, d.p, total * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
  return la_sync_and_check(ctx, "qr extract");
}

}  // namespace

// ---- C ABI -----------------------------------------------------------------

la_status la_qr_new(la_ctx ctx, const double* a, size_t m, size_t n, la_qr* out) {
  LA_TRY(qr_check_ctx(ctx));
  if (!a || !out) return LA_INVALID;
  *out = nullptr;
  la_qr h = nullptr;
  LA_TRY(qr_alloc(ctx, m, n, &h));
  cudaError_t e = cudaMemcpy2DAsync(h->d_qr, h->ld * sizeof(double), a, n * sizeof(double),
                                    n * sizeof(double), m, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) {
    la_qr_free(h);
    return la_cuda_fail(ctx, e, "copy A to device");
  }
  return qr_new_common(ctx, h, out);
}

la_status la_qr_new_device(la_ctx ctx, const double* d_a, size_t lda, size_t m, size_t n,
                           la_qr* out) {
  LA_TRY(qr_check_ctx(ctx));
  if (!d_a || !out || lda < n) return LA_INVALID;
  *out = nullptr;
  la_qr h = nullptr;
  LA_TRY(qr_alloc(ctx, m, n, &h));
  cudaError_t e = cudaMemcpy2DAsync(h->d_qr, h->ld * sizeof(double), d_a, lda * sizeof(double),
                                    n * sizeof(double), m, cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) {
    la_qr_free(h);
    return la_cuda_fail(ctx, e, "copy A on device");
  }
  return qr_new_common(ctx, h, out);
}

void la_qr_free(la_qr h) {
  if (!h) return;
  cudaSetDevice(h->ctx->device);
  la_device_free(h->ctx, h->d_qr);
  la_device_free(h->ctx, h->d_rdiag);
  la_device_free(h->ctx, h->d_gram);
  delete h;
}

la_status la_qr_is_full_rank(la_qr h, int* out) {
  if (!h || !out) return LA_INVALID;
  return qr_full_rank(h, out);
}

la_status la_qr_get_r(la_qr h, double* out) {
  if (!h || !out) return LA_INVALID;
  return qr_extract_host(h, 0, out);
}

la_status la_qr_get_h(la_qr h, double* out) {
  if (!h || !out) return LA_INVALID;
  return qr_extract_host(h, 1, out);
}

la_status la_qr_get_q(la_qr h, double* out) {
  if (!h || !out) return LA_INVALID;
  la_ctx ctx = h->ctx;
  LA_TRY(qr_check_ctx(ctx));
  const int m = (int)h->m, n = (int)h->n, dc = std::min(m, n);
  const bool exact = h->arith == LA_ARITH_EXACT;
  const size_t ldq = pad4q(h->m);
  QBuf Qm(ctx);
  LA_TRY(Qm.alloc(h->m * ldq * sizeof(double)));
  qr_q_init_kernel<<<blocks_for(h->m * h->m, 256), 256, 0, ctx->stream>>>(Qm.d(), ldq, m, dc);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "qr_q_init_kernel"));
  if (h->d_gram)  // blocked FAST factorization: the reflections block by block
    LA_TRY(qr_blocked_apply(ctx, h->d_qr, h->ld, m, dc, h->d_rdiag, h->d_gram, 1, Qm.d(), ldq, m));
  else
    for (int k = dc - 1; k >= 0; k--)  // qr.rs:163-191
      LA_TRY(reflect(ctx, exact, h->d_qr, h->ld, k, k, m, h->d_rdiag, Qm.d(), ldq, k, m, 1));
  LA_CUDA(ctx, cudaMemcpy2DAsync(out, h->m * sizeof(double), Qm.p, ldq * sizeof(double),
                                 h->m * sizeof(double), h->m, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  return la_sync_and_check(ctx, "la_qr_get_q");
}

la_status la_qr_solve(la_qr h, const double* b, size_t brows, size_t nrhs, double* x) {
  if (!h || !b || !x) return LA_INVALID;
  la_ctx ctx = h->ctx;
  LA_TRY(qr_check_ctx(ctx));
  if (brows != h->m || nrhs == 0) return LA_BADSHAPE;  // qr.rs:200
  int fr = 0;
  LA_TRY(qr_full_rank(h, &fr));  // LA_BADSHAPE past rdiag (n > m)
  if (!fr) return LA_SINGULAR;   // qr.rs:201-203: None
  if (h->m != h->n) return LA_BADSHAPE;  // Matrix::new(n, nx, m * nx values) (qr.rs:237)
  const int n = (int)h->n, nx = (int)nrhs;
  const bool exact = h->arith == LA_ARITH_EXACT;
  const size_t ldw = pad4q(nrhs), ldr = pad4q(h->n);
  QBuf X(ctx), R(ctx);
  LA_TRY(X.alloc(h->n * ldw * sizeof(double)));
  LA_TRY(R.alloc(h->n * ldr * sizeof(double)));
  LA_CUDA(ctx, cudaMemcpy2DAsync(X.p, ldw * sizeof(double), b, nrhs * sizeof(double),
                                 nrhs * sizeof(double), h->n, cudaMemcpyHostToDevice,
                                 ctx->stream));
  if (h->d_gram)  // Y = Q' B (qr.rs:211-223), block by block
    LA_TRY(qr_blocked_apply(ctx, h->d_qr, h->ld, n, n, h->d_rdiag, h->d_gram, 2, X.d(), ldw, nx));
  else
    for (int k = 0; k < n; k++)  // Y = Q' B (qr.rs:211-223)
      LA_TRY(reflect(ctx, exact, h->d_qr, h->ld, k, k, n, h->d_rdiag, X.d(), ldw, 0, nx, 2));
  qr_extract_kernel<<<blocks_for(h->n * h->n, 256), 256, 0, ctx->stream>>>(
      h->d_qr, h->ld, h->d_rdiag, n, n, R.d(), ldr, 0);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "qr_extract_kernel"));
  // R X = Y (qr.rs:225-235): descending terms, then the division by rdiag
  LA_TRY(launch_tri_wave(ctx, exact, true, true, R.d(), ldr, X.d(), ldw, n, nx));
  LA_CUDA(ctx, cudaMemcpy2DAsync(x, nrhs * sizeof(double), X.p, ldw * sizeof(double),
                                 nrhs * sizeof(double), h->n, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  return la_sync_and_check(ctx, "la_qr_solve");
}

// Matrix::pinverse (mod.rs:1049-1057): (R' R)^-1 A' through the library's QR,
// Mul (mod.rs:957-980) and inverse (LU, mod.rs:1034-1037); the transposes
// (Matrix::t, mod.rs:653-666) are copies on the host, as in the reference.
// LA_BADSHAPE where inverse() is None and unwrap panics.
la_status la_matrix_pinverse(la_ctx ctx, const double* a, size_t m, size_t n, double* out) {
  LA_TRY(qr_check_ctx(ctx));
  if (!a || !out) return LA_INVALID;
  la_qr h = nullptr;
  LA_TRY(la_qr_new(ctx, a, m, n, &h));
  std::vector<double> r(m * n), rt(n * m), rtr(n * n), inv(n * n), at(n * m);
  la_status s = la_qr_get_r(h, r.data());
  la_qr_free(h);
  if (s != LA_OK) return s;
  for (size_t i = 0; i < m; i++)
    for (size_t j = 0; j < n; j++) {
      rt[j * m + i] = r[i * n + j];
      at[j * m + i] = a[i * n + j];
    }
  LA_TRY(la_matrix_mul(ctx, rt.data(), n, m, r.data(), m, n, rtr.data()));
  s = la_matrix_inverse(ctx, rtr.data(), n, n, inv.data());
  if (s == LA_SINGULAR) return LA_BADSHAPE;  // .inverse().unwrap()
  LA_TRY(s);
  return la_matrix_mul(ctx, inv.data(), n, n, at.data(), n, m, out);
}
