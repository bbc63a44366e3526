// Cholesky decomposition of a symmetric positive definite matrix
// (CholeskyDecomposition, src/decomp/cholesky.rs:56-145): A = L L'.
//
// The reference computes L one row at a time (cholesky.rs:64-107): for row j
// and k < j, L[j][k] = (A[j][k] - s) / L[k][k] with s the sum of
// L[k][i] L[j][i] over i < k, added in ascending i; the diagonal
// L[j][j] = sqrt(A[j][j] - d) with d the sum of L[j][k]^2 in ascending k. It
// returns None for a non-square matrix, at the first pair with
// A[k][j] != A[j][k], or at the first d <= 0.
//
// Here the same values come from a blocked right-looking form in 64-column
// panels (no pivoting, so every panel step is known in advance):
//   1. chol_sym_check_kernel compares every strictly lower entry with its
//      upper twin (the reference's '!=', so NaN fails), before anything is
//      written;
//   2. chol_diag_kernel factors the 64 x 64 diagonal block on one CTA, column
//      by column;
//   3. chol_panel_kernel computes the rows below it, one thread per row with
//      the row's 64 values in registers;
//   4. the trailing update A22 -= L21 L21' runs on the FP64 GEMM (TMA tiles in
//      FAST) over row strips, each strip only up to its own diagonal, so about
//      half of the square is skipped.
// FAST accumulates A - sum with FMA in place. EXACT keeps, per element, the
// running sum s in a second array S, adds products unfused in ascending i (the
// GEMM's EXACT_ADD mode, then the panel kernels) and forms (A - s) / L[k][k]
// and sqrt(A - d) exactly as the reference does, so L is bit-identical to it.
// A None result is reported after the whole factorization: the reference stops
// at the first failing row, and every such row fails here too.
#include "la_internal.cuh"

struct la_chol_handle {
  la_ctx ctx = nullptr;
  size_t n = 0, ld = 0;
  double* d_l = nullptr;   // L, n x n with pitch ld, zeros above the diagonal
  double* d_lt = nullptr;  // L' (built on the first FAST solve)
  int arith = LA_ARITH_FAST;
};

namespace {

constexpr int CHW = 64;   // panel width
constexpr int CHP = CHW + 1;
constexpr int PANEL_T = 64;  // two warps per CTA: rows spread over more SMs

size_t pad4c(size_t x) { return (x + 3) & ~size_t(3); }

struct Buf {
  la_ctx ctx;
  void* p = nullptr;
  explicit Buf(la_ctx c) : ctx(c) {}
  ~Buf() { la_device_free(ctx, p); }
  la_status alloc(size_t bytes) { return la_device_alloc(ctx, &p, bytes); }
  double* d() { return static_cast<double*>(p); }
};

// flags[0] |= 1 when some strictly lower entry differs from its upper twin
// (cholesky.rs:89-91). One 32 x 32 tile pair per CTA, lower tiles only.
__global__ void chol_sym_check_kernel(const double* __restrict__ A, size_t ld, int n, int* flags) {
  __shared__ double t[32][33];
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj > bi) return;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  // t[c][r] = A[bj*32 + r][bi*32 + c]: the upper twin tile, transposed
  for (int r = ty; r < 32; r += 8) {
    const int gr = bj * 32 + r, gc = bi * 32 + tx;
    t[tx][r] = (gr < n && gc < n) ? A[(size_t)gr * ld + gc] : 0.0;
  }
  __syncthreads();
  int bad = 0;
  for (int r = ty; r < 32; r += 8) {
    const int gr = bi * 32 + r, gc = bj * 32 + tx;
    if (gr < n && gc < n && gr > gc && A[(size_t)gr * ld + gc] != t[r][tx]) bad = 1;
  }
  if (__syncthreads_or(bad) && tx == 0 && ty == 0) atomicOr(flags, 1);
}

// Diagonal block [j0, j0 + jb)^2 on one CTA (lower part, diagonal included).
// flags[1] |= 1 at a non-positive d (cholesky.rs:97-100; NaN is not <= 0).
template <bool EXACT>
__global__ void __launch_bounds__(256)
chol_diag_kernel(double* L, double* S, size_t ld, int j0, int jb, int* flags) {
  extern __shared__ __align__(16) double chd_raw[];
  double(*a)[CHP] = reinterpret_cast<double(*)[CHP]>(chd_raw);
  double(*s)[CHP] = reinterpret_cast<double(*)[CHP]>(chd_raw + CHW * CHP);
  const int tid = threadIdx.x;
  for (int idx = tid; idx < jb * jb; idx += 256) {
    const int r = idx / jb, c = idx % jb;
    if (c <= r) {
      a[r][c] = L[(size_t)(j0 + r) * ld + j0 + c];
      if (EXACT) s[r][c] = S[(size_t)(j0 + r) * ld + j0 + c];
    }
  }
  __syncthreads();
  for (int k = 0; k < jb; k++) {
    if (tid == 0) {
      const double d = EXACT ? __dsub_rn(a[k][k], s[k][k]) : a[k][k];  // :96
      if (d <= 0.0) atomicOr(flags + 1, 1);
      a[k][k] = sqrt(d);  // :101
    }
    __syncthreads();
    const double dk = a[k][k];
    for (int r = k + 1 + tid; r < jb; r += 256)
      a[r][k] = EXACT ? __dsub_rn(a[r][k], s[r][k]) / dk : a[r][k] / dk;  // :82
    __syncthreads();
    const int m = jb - k - 1;
    for (int idx = tid; idx < m * m; idx += 256) {
      const int r = k + 1 + idx / m, c = k + 1 + idx % m;
      if (c > r) continue;
      if (EXACT) s[r][c] = __dadd_rn(s[r][c], __dmul_rn(a[r][k], a[c][k]));  // :78, :86
      else a[r][c] = fma(-a[r][k], a[c][k], a[r][c]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < jb * jb; idx += 256) {
    const int r = idx / jb, c = idx % jb;
    if (c <= r) L[(size_t)(j0 + r) * ld + j0 + c] = a[r][c];
  }
}

// FAST form of the diagonal block: warp 0 takes the square root and scales
// the column by its reciprocal, then all threads apply the rank-1 update to
// the lower triangle still open (rows and columns from a 16 x 16 thread
// grid, no index division); two barriers per column.
__global__ void __launch_bounds__(256)
chol_diag_fast_kernel(double* L, size_t ld, int j0, int jb, int* flags) {
  extern __shared__ __align__(16) double chd_raw[];
  double(*a)[CHP] = reinterpret_cast<double(*)[CHP]>(chd_raw);
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int idx = tid; idx < jb * jb; idx += 256) {
    const int r = idx / jb, c = idx % jb;
    if (c <= r) a[r][c] = L[(size_t)(j0 + r) * ld + j0 + c];
  }
  __syncthreads();
  for (int k = 0; k < jb; k++) {
    if (tid < 32) {
      const double d = a[k][k];
      const double q = sqrt(d);
      const double rq = 1.0 / q;
      if (tid == 0) {
        if (d <= 0.0) atomicOr(flags + 1, 1);  // cholesky.rs:97-100
        a[k][k] = q;
      }
      for (int r = k + 1 + tid; r < jb; r += 32) a[r][k] *= rq;
    }
    __syncthreads();
    for (int r = k + 1 + ty; r < jb; r += 16) {
      const double lr = a[r][k];
      for (int c = k + 1 + tx; c <= r; c += 16) a[r][c] = fma(-lr, a[c][k], a[r][c]);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < jb * jb; idx += 256) {
    const int r = idx / jb, c = idx % jb;
    if (c <= r) L[(size_t)(j0 + r) * ld + j0 + c] = a[r][c];
  }
}

// Rows [r0, n) of the panel's columns [j0, j0 + 64): one thread per row, the
// row's running values (FAST: A - sum; EXACT: the sums s) in registers, the
// finished diagonal block broadcast from shared memory. Only a full-width
// panel has rows below it (a narrower one is the last), so the width is fixed.
template <bool EXACT>
__global__ void __launch_bounds__(PANEL_T)
chol_panel_kernel(double* L, const double* S, size_t ld, int j0, int r0, int n) {
  __shared__ double dg[CHW][CHP];
  __shared__ double rdg[CHW];
  for (int idx = threadIdx.x; idx < CHW * CHW; idx += PANEL_T) {
    const int r = idx / CHW, c = idx % CHW;
    if (c <= r) dg[r][c] = L[(size_t)(j0 + r) * ld + j0 + c];
  }
  __syncthreads();
  if (!EXACT && threadIdx.x < CHW) rdg[threadIdx.x] = 1.0 / dg[threadIdx.x][threadIdx.x];
  __syncthreads();
  const int r = r0 + blockIdx.x * PANEL_T + threadIdx.x;
  if (r >= n) return;
  double* row = L + (size_t)r * ld + j0;
  double v[CHW];
#pragma unroll
  for (int c = 0; c < CHW; c++) v[c] = EXACT ? S[(size_t)r * ld + j0 + c] : row[c];
#pragma unroll
  for (int k = 0; k < CHW; k++) {
    const double x = EXACT ? __dsub_rn(row[k], v[k]) / dg[k][k] : v[k] * rdg[k];  // :82
    row[k] = x;
#pragma unroll
    for (int c = k + 1; c < CHW; c++)
      v[c] = EXACT ? __dadd_rn(v[c], __dmul_rn(x, dg[c][k])) : fma(-x, dg[c][k], v[c]);
  }
}

// T[k][c] = L[r0 + c][j0 + k]: the panel's rows below the diagonal block,
// transposed, as the GEMM's K x N operand.
__global__ void chol_transpose_kernel(const double* __restrict__ L, size_t ld, int j0, int jb,
                                      int r0, int ncols, double* T, size_t ldt) {
  __shared__ double t[32][33];
  const int c0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int i = ty; i < 32; i += 8) {
    const int c = c0 + i, k = k0 + tx;
    t[i][tx] = (c < ncols && k < jb) ? L[(size_t)(r0 + c) * ld + j0 + k] : 0.0;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int k = k0 + i, c = c0 + tx;
    if (k < jb && c < ncols) T[(size_t)k * ldt + c] = t[tx][i];
  }
}

// L[r][c] = 0 for c > r (cholesky.rs:104-106).
__global__ void chol_zero_upper_kernel(double* L, size_t ld, int n) {
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj < bi) return;
  for (int r = bi * 32 + threadIdx.y; r < min(n, bi * 32 + 32); r += 8) {
    const int c = bj * 32 + threadIdx.x;
    if (c < n && c > r) L[(size_t)r * ld + c] = 0.0;
  }
}

// L' X = Y with the reference's term order (cholesky.rs:133-141): row k takes
// x_i l_ik for i = k+1 .. n-1 ascending, unfused, then divides by l_kk. Each
// row waits for its nearest neighbour first, so the order admits no
// wavefront; one thread per right-hand side runs the whole sweep (EXACT only).
__global__ void chol_back_exact_kernel(const double* __restrict__ L, size_t ld, double* X,
                                       size_t ldx, int n, int nrhs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nrhs) return;
  for (int k = n - 1; k >= 0; k--) {
    double s = X[(size_t)k * ldx + j];
    for (int i = k + 1; i < n; i++)
      s = __dsub_rn(s, __dmul_rn(X[(size_t)i * ldx + j], L[(size_t)i * ld + k]));
    X[(size_t)k * ldx + j] = s / L[(size_t)k * ld + k];
  }
}

cudaError_t configure_chol() {
  static la_device_once once;
  return once.run([](int) {
    cudaError_t e = cudaFuncSetAttribute(chol_diag_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(2 * CHW * CHP * sizeof(double)));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(chol_diag_fast_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(CHW * CHP * sizeof(double)));
    return e;
  });
}

la_status chol_check_ctx(la_ctx ctx) {
  if (!ctx) return LA_INVALID;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaSetDevice");
  return LA_OK;
}

// Factors h->d_l (a copy of A) in place; *none = the reference's None.
la_status chol_factor(la_ctx ctx, la_chol h, int* none) {
  const int n = (int)h->n;
  const size_t ld = h->ld;
  const bool exact = h->arith == LA_ARITH_EXACT;
  double* L = h->d_l;
  cudaStream_t st = ctx->stream;
  LA_CUDA(ctx, configure_chol());
  int* d_flags = reinterpret_cast<int*>(ctx->d_small);
  LA_CUDA(ctx, cudaMemsetAsync(d_flags, 0, 2 * sizeof(int), st));
  const int nt = (n + 31) / 32;
  chol_sym_check_kernel<<<dim3(nt, nt), dim3(32, 8), 0, st>>>(L, ld, n, d_flags);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "chol_sym_check_kernel"));

  Buf S(ctx), T0(ctx), T1(ctx);
  if (exact) {
    LA_TRY(S.alloc((size_t)n * ld * sizeof(double)));
    LA_CUDA(ctx, cudaMemsetAsync(S.p, 0, (size_t)n * ld * sizeof(double), st));
  }
  // Transposed panels (the GEMM's K x N operand), two so that panel k + 1 can
  // be transposed while panel k's update still reads its own.
  const size_t ldt = pad4c((size_t)n);
  if (n > CHW) {
    LA_TRY(T0.alloc((size_t)CHW * ldt * sizeof(double)));
    LA_TRY(T1.alloc((size_t)CHW * ldt * sizeof(double)));
  }
  double* Tbuf[2] = {T0.d(), T1.d()};
  const size_t dsm = (exact ? 2 : 1) * CHW * CHP * sizeof(double);
  const bool look = ctx->lookahead != 0 && ctx->side_stream != nullptr;

  // Diagonal block, rows below and transpose of panel [j0, j0 + jb) on stream s.
  auto panel = [&](int j0, int jb, double* T, cudaStream_t s) -> la_status {
    const int j1 = j0 + jb;
    if (exact)
      chol_diag_kernel<true><<<1, 256, dsm, s>>>(L, S.d(), ld, j0, jb, d_flags);
    else
      chol_diag_fast_kernel<<<1, 256, dsm, s>>>(L, ld, j0, jb, d_flags);
    ctx->launches++;
    LA_TRY(la_check_launch(ctx, "chol_diag_kernel"));
    if (j1 >= n) return LA_OK;
    const int rows = n - j1;
    const int pg = (rows + PANEL_T - 1) / PANEL_T;
    if (exact)
      chol_panel_kernel<true><<<pg, PANEL_T, 0, s>>>(L, S.d(), ld, j0, j1, n);
    else
      chol_panel_kernel<false><<<pg, PANEL_T, 0, s>>>(L, nullptr, ld, j0, j1, n);
    ctx->launches++;
    LA_TRY(la_check_launch(ctx, "chol_panel_kernel"));
    chol_transpose_kernel<<<dim3((rows + 31) / 32, (jb + 31) / 32), dim3(32, 8), 0, s>>>(
        L, ld, j0, jb, j1, rows, T, ldt);
    ctx->launches++;
    return la_check_launch(ctx, "chol_transpose_kernel");
  };
  // A22 -= L21 L21' (EXACT: S22 += ...) of panel [j0, j0 + jb) on rows and
  // columns >= c0 (lower part): FAST as one launch over the tiles at or below
  // the diagonal; EXACT (and FAST where TMA cannot take the operands) in up
  // to 8 row strips [a, b) that each stop at their own diagonal block.
  auto update = [&](int j0, int jb, const double* T, int c0) -> la_status {
    const int j1 = j0 + jb, rows = n - c0;
    if (rows <= 0) return LA_OK;
    if (!exact) {
      const la_status r = launch_gemm_lower(ctx, rows, jb, L + (size_t)c0 * ld + j0, ld,
                                            T + (c0 - j1), ldt, L + (size_t)c0 * ld + c0, ld);
      if (r != LA_UNSUPPORTED) return r;
    }
    const int nstrip = std::max(1, std::min(8, rows / 512));
    const int hs = ((rows + nstrip - 1) / nstrip + CHW - 1) / CHW * CHW;
    for (int a = c0; a < n; a += hs) {
      const int b = std::min(n, a + hs);
      double* C = (exact ? S.d() : L) + (size_t)a * ld + c0;
      LA_TRY(launch_gemm(ctx, exact ? GM_EXACT_ADD : GM_FMA_SUB, b - a, b - c0, jb,
                         L + (size_t)a * ld + j0, ld, T + (c0 - j1), ldt, C, ld));
    }
    return LA_OK;
  };
  // The next panel's columns [j1, j2) of rows >= j1 (a plain GEMM).
  auto update_next = [&](int j0, int jb, const double* T, int j1, int j2) -> la_status {
    double* C = (exact ? S.d() : L) + (size_t)j1 * ld + j1;
    return launch_gemm(ctx, exact ? GM_EXACT_ADD : GM_FMA_SUB, n - j1, j2 - j1, jb,
                       L + (size_t)j1 * ld + j0, ld, T, ldt, C, ld);
  };

  // Lookahead, as in the LU: panel k's update of panel k + 1's columns first,
  // then panel k + 1 on the high-priority side stream while the rest of panel
  // k's update runs (rows and columns >= j2). They touch disjoint data: panel
  // k + 1 owns columns [j1, j2) of rows >= j1, and the rest of the update reads
  // panel k's finished columns and its transposed copy. The update keeps its
  // full occupancy (an earlier form that capped it at two CTAs per SM to leave
  // the panel room measured slower than no lookahead at all).
  LA_TRY(panel(0, std::min(CHW, n), Tbuf[0], st));
  for (int j0 = 0, k = 0; j0 < n; j0 += CHW, k++) {
    const int jb = std::min(CHW, n - j0), j1 = j0 + jb;
    if (j1 >= n) break;
    const int jbn = std::min(CHW, n - j1), j2 = j1 + jbn;
    double* Tk = Tbuf[k & 1];
    double* Tn = Tbuf[(k + 1) & 1];
    if (look && j2 < n) {
      LA_TRY(update_next(j0, jb, Tk, j1, j2));
      LA_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
      LA_CUDA(ctx, cudaStreamWaitEvent(ctx->side_stream, ctx->ev_fork, 0));
      LA_TRY(panel(j1, jbn, Tn, ctx->side_stream));
      LA_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->side_stream));
      LA_TRY(update(j0, jb, Tk, j2));
      LA_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_join, 0));
    } else {
      LA_TRY(update(j0, jb, Tk, j1));
      LA_TRY(panel(j1, jbn, Tn, st));
    }
  }
  chol_zero_upper_kernel<<<dim3(nt, nt), dim3(32, 8), 0, st>>>(L, ld, n);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "chol_zero_upper_kernel"));
  int* flags = static_cast<int*>(ctx->h_pinned);
  LA_CUDA(ctx, cudaMemcpyAsync(flags, d_flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
  LA_TRY(la_sync_and_check(ctx, "cholesky factorization"));
  *none = (flags[0] | flags[1]) != 0;
  return LA_OK;
}

la_status chol_alloc(la_ctx ctx, size_t n, la_chol* out) {
  if (n > (size_t)INT32_MAX / 2) return LA_UNSUPPORTED;
  la_chol h = new (std::nothrow) la_chol_handle();
  if (!h) return LA_NOMEM;
  h->ctx = ctx;
  h->n = n;
  h->ld = pad4c(n);
  h->arith = ctx->arith;
  void* p = nullptr;
  la_status s = la_device_alloc(ctx, &p, n * h->ld * sizeof(double));
  if (s != LA_OK) { delete h; return s; }
  h->d_l = static_cast<double*>(p);
  *out = h;
  return LA_OK;
}

la_status chol_new_common(la_ctx ctx, la_chol h, la_chol* out) {
  int none = 0;
  la_status s = chol_factor(ctx, h, &none);
  if (s == LA_OK && none) s = LA_SINGULAR;
  if (s != LA_OK) {
    la_chol_free(h);
    return s;
  }
  *out = h;
  return LA_OK;
}

la_status chol_solve_device_common(la_chol h, const double* d_b, size_t ldb, size_t brows,
                                   size_t nrhs, double* d_x, size_t ldx) {
  la_ctx ctx = h->ctx;
  if (brows != h->n) return LA_BADSHAPE;  // cholesky.rs:118
  if (nrhs == 0) return LA_BADSHAPE;      // Matrix::new asserts cols > 0
  const int n = (int)h->n;
  const bool exact = h->arith == LA_ARITH_EXACT;
  cudaStream_t st = ctx->stream;
  const size_t ldw = pad4c(nrhs);
  Buf X(ctx);
  LA_TRY(X.alloc(h->n * ldw * sizeof(double)));
  LA_CUDA(ctx, cudaMemcpy2DAsync(X.p, ldw * sizeof(double), d_b, ldb * sizeof(double),
                                 nrhs * sizeof(double), h->n, cudaMemcpyDeviceToDevice, st));
  // L Y = B (cholesky.rs:123-131): ascending terms, then the division
  LA_TRY(launch_tri_wave(ctx, exact, false, true, h->d_l, h->ld, X.d(), ldw, n, (int)nrhs));
  if (exact) {
    chol_back_exact_kernel<<<((int)nrhs + 127) / 128, 128, 0, st>>>(h->d_l, h->ld, X.d(), ldw, n,
                                                                   (int)nrhs);
    ctx->launches++;
    LA_TRY(la_check_launch(ctx, "chol_back_exact_kernel"));
  } else {
    // L' X = Y on the transposed copy (rows of L' contiguous), any term order
    if (!h->d_lt) {
      void* p = nullptr;
      LA_TRY(la_device_alloc(ctx, &p, h->n * h->ld * sizeof(double)));
      h->d_lt = static_cast<double*>(p);
      const int nt = (n + 31) / 32;
      chol_transpose_kernel<<<dim3(nt, nt), dim3(32, 8), 0, st>>>(h->d_l, h->ld, 0, n, 0, n,
                                                                  h->d_lt, h->ld);
      ctx->launches++;
      LA_TRY(la_check_launch(ctx, "chol_transpose_kernel"));
    }
    LA_TRY(launch_tri_wave(ctx, false, true, true, h->d_lt, h->ld, X.d(), ldw, n, (int)nrhs));
  }
  LA_CUDA(ctx, cudaMemcpy2DAsync(d_x, ldx * sizeof(double), X.p, ldw * sizeof(double),
                                 nrhs * sizeof(double), h->n, cudaMemcpyDeviceToDevice, st));
  return LA_OK;
}

}  // namespace

// ---- C ABI -----------------------------------------------------------------

la_status la_chol_new(la_ctx ctx, const double* a, size_t m, size_t n, la_chol* out) {
  LA_TRY(chol_check_ctx(ctx));
  if (!a || !out) return LA_INVALID;
  *out = nullptr;
  if (m == 0 || n == 0) return LA_BADSHAPE;  // Matrix::new asserts (mod.rs:209)
  if (m != n) return LA_SINGULAR;           // cholesky.rs:57-59: None
  la_chol h = nullptr;
  LA_TRY(chol_alloc(ctx, n, &h));
  cudaError_t e = cudaMemcpy2DAsync(h->d_l, h->ld * sizeof(double), a, n * sizeof(double),
                                    n * sizeof(double), n, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) {
    la_chol_free(h);
    return la_cuda_fail(ctx, e, "copy A to device");
  }
  return chol_new_common(ctx, h, out);
}

la_status la_chol_new_device(la_ctx ctx, const double* d_a, size_t lda, size_t n, la_chol* out) {
  LA_TRY(chol_check_ctx(ctx));
  if (!d_a || !out || lda < n) return LA_INVALID;
  *out = nullptr;
  if (n == 0) return LA_BADSHAPE;
  la_chol h = nullptr;
  LA_TRY(chol_alloc(ctx, n, &h));
  cudaError_t e = cudaMemcpy2DAsync(h->d_l, h->ld * sizeof(double), d_a, lda * sizeof(double),
                                    n * sizeof(double), n, cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) {
    la_chol_free(h);
    return la_cuda_fail(ctx, e, "copy A on device");
  }
  return chol_new_common(ctx, h, out);
}

void la_chol_free(la_chol h) {
  if (!h) return;
  cudaSetDevice(h->ctx->device);
  la_device_free(h->ctx, h->d_l);
  la_device_free(h->ctx, h->d_lt);
  delete h;
}

la_status la_chol_n(la_chol h, size_t* n) {
  if (!h || !n) return LA_INVALID;
  *n = h->n;
  return LA_OK;
}

la_status la_chol_get_l(la_chol h, double* out) {
  if (!h || !out) return LA_INVALID;
  la_ctx ctx = h->ctx;
  LA_TRY(chol_check_ctx(ctx));
  LA_CUDA(ctx, cudaMemcpy2DAsync(out, h->n * sizeof(double), h->d_l, h->ld * sizeof(double),
                                 h->n * sizeof(double), h->n, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  return la_sync_and_check(ctx, "la_chol_get_l");
}

la_status la_chol_solve(la_chol h, const double* b, size_t brows, size_t nrhs, double* x) {
  if (!h || !b || !x) return LA_INVALID;
  la_ctx ctx = h->ctx;
  LA_TRY(chol_check_ctx(ctx));
  if (brows != h->n || nrhs == 0) return LA_BADSHAPE;
  Buf B(ctx);
  LA_TRY(B.alloc(brows * nrhs * sizeof(double)));
  LA_CUDA(ctx, cudaMemcpyAsync(B.p, b, brows * nrhs * sizeof(double), cudaMemcpyHostToDevice,
                               ctx->stream));
  LA_TRY(chol_solve_device_common(h, B.d(), nrhs, brows, nrhs, B.d(), nrhs));
  LA_CUDA(ctx, cudaMemcpyAsync(x, B.p, brows * nrhs * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
  return la_sync_and_check(ctx, "la_chol_solve");
}

la_status la_chol_solve_device(la_chol h, const double* d_b, size_t ldb, size_t brows,
                               size_t nrhs, double* d_x, size_t ldx) {
  if (!h || !d_b || !d_x || ldb < nrhs || ldx < nrhs) return LA_INVALID;
  LA_TRY(chol_check_ctx(h->ctx));
  return chol_solve_device_common(h, d_b, ldb, brows, nrhs, d_x, ldx);
}
