// C-ABI entry points of the LU path: LUDecomposition::{new, solve, det, ...},
// Matrix::{det, solve, inverse, is_non_singular} and Matrix * Matrix.
//
// Blocked right-looking LU (panel width W, default 64), for each panel
// [j0, j1 = j0 + jb):
//   panel  : cooperative kernel, pivots + L21/U11 of the panel (lu_panel.cu)
//   laswp  : the panel's row swaps on the other columns (lu.rs:140-145)
//   trsm   : U12 = L11^{-1} A12 for rows [j0, j1)
//   gemm   : A22 -= L21 * U12 (FAST) or S22 += L21 * U12 (EXACT carry)
// In EXACT mode S holds, for every not-yet-finished element, the partial sum
// of lu.rs:124-126 over the k already processed, so each element's sum is
// formed in the reference's order and subtracted once (lu.rs:128).
#include <algorithm>
#include <cstring>
#include <vector>

#include "la_internal.cuh"

namespace {

size_t pad4(size_t x) { return (x + 3) & ~size_t(3); }
bool aligned16(const void* p, size_t ld) {
  return (reinterpret_cast<uintptr_t>(p) % 16 == 0) && (ld % 2 == 0);
}

struct DevBuf {
  la_ctx ctx;
  void* p = nullptr;
  explicit DevBuf(la_ctx c) : ctx(c) {}
  ~DevBuf() { la_device_free(ctx, p); }
  la_status alloc(size_t bytes) { return la_device_alloc(ctx, &p, bytes); }
  double* d() { return static_cast<double*>(p); }
};

// Phase timing for LA_OPT_PROFILE: a pair of events (from the context's pool)
// around each phase instance on the stream it runs on; the per-category sums
// are device time, so a panel overlapped with the trailing update is counted
// in full in both categories.
struct PhaseTimer {
  la_ctx ctx;
  bool on;
  size_t used = 0;
  struct Span { size_t b, e; int cat; };
  std::vector<Span> spans;
  explicit PhaseTimer(la_ctx c) : ctx(c), on(c->profile != 0) {}
  size_t record(cudaStream_t s) {
    if (used == ctx->event_pool.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) { on = false; return 0; }
      ctx->event_pool.push_back(e);
    }
    cudaEventRecord(ctx->event_pool[used], s);
    return used++;
  }
  size_t begin(cudaStream_t s) { return on ? record(s) : 0; }
  void end(cudaStream_t s, size_t b, int cat) {
    if (!on) return;
    size_t e = record(s);
    if (on) spans.push_back({b, e, cat});
  }
  void finish() {
    for (int i = 0; i < 5; i++) ctx->phase_ms[i] = 0;
    if (!on) return;
    for (auto& sp : spans) {
      cudaEventSynchronize(ctx->event_pool[sp.e]);
      float ms = 0;
      cudaEventElapsedTime(&ms, ctx->event_pool[sp.b], ctx->event_pool[sp.e]);
      ctx->phase_ms[sp.cat] += ms;
    }
  }
};

enum { PH_PANEL = 0, PH_SWAP = 1, PH_TRSM = 2, PH_GEMM = 3, PH_OTHER = 4 };

// Shared memory that keeps trailing-update GEMM CTAs at two per SM, leaving an
// SM room for one CTA of the concurrent panel kernel.
constexpr size_t GEMM_SMEM_WITH_PANEL = 78 * 1024;

// Factors h->d_lu in place.
//
// With lookahead (default), after panel p's row swaps and triangular update,
// the columns of panel p+1 get their trailing update first; panel p+1 is then
// factored on the high-priority side stream while the rest of panel p's
// trailing update runs on the main stream. The two touch disjoint columns:
// panel p+1 owns columns [j1, j2) of rows >= j1, the rest of the update writes
// columns >= j2 and reads L21 (columns < j1) and U12 (rows < j1).
}  // namespace

la_status lu_factor_enqueue(la_ctx ctx, la_lu h, int* d_flags) {
  const bool exact = (h->arith == LA_ARITH_EXACT);
  const int m = (int)h->m, n = (int)h->n;
  const size_t ld = h->ld;
  const int kmin = std::min(m, n);
  const int W = ctx->panel_width;
  const bool look = ctx->lookahead != 0;
  cudaStream_t ms = ctx->stream, ss = ctx->side_stream;
  double* A = h->d_lu;
  DevBuf S(ctx);
  if (exact) {
    LA_TRY(S.alloc((size_t)m * ld * sizeof(double)));
    LA_CUDA(ctx, cudaMemsetAsync(S.p, 0, (size_t)m * ld * sizeof(double), ms));
  }
  LA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(unsigned), ms));
  unsigned bar_base = 0;
  PhaseTimer t(ctx);
  const int gmode = exact ? GM_EXACT_ADD : GM_FMA_SUB;
  auto trailing = [&](int j0, int jb, int c0, int c1, size_t min_smem) -> la_status {
    // rows [j0+jb, m), columns [c0, c1)
    const int j1 = j0 + jb;
    if (j1 >= m || c1 <= c0) return LA_OK;
    const double* L21 = A + (size_t)j1 * ld + j0;
    const double* U12 = A + (size_t)j0 * ld + c0;
    double* C = exact ? S.d() + (size_t)j1 * ld + c0 : A + (size_t)j1 * ld + c0;
    size_t b = t.begin(ms);
    la_status st = launch_gemm(ctx, gmode, m - j1, c1 - c0, jb, L21, ld, U12, ld, C, ld, min_smem);
    t.end(ms, b, PH_GEMM);
    return st;
  };

  {
    size_t b = t.begin(ms);
    LA_TRY(launch_panel(ctx, ms, exact, A, S.d(), ld, m, 0, std::min(W, kmin), h->d_ipiv,
                        &bar_base));
    t.end(ms, b, PH_PANEL);
  }
  for (int j0 = 0; j0 < kmin; j0 += W) {
    const int jb = std::min(W, kmin - j0);
    const int j1 = j0 + jb;
    size_t b = t.begin(ms);
    LA_TRY(launch_laswp(ctx, exact, A, S.d(), ld, n, j0, jb));
    t.end(ms, b, PH_SWAP);
    if (j1 < n) {
      b = t.begin(ms);
      LA_TRY(launch_trsm_rowpanel(ctx, exact, A, S.d(), ld, j0, jb, j1, n));
      t.end(ms, b, PH_TRSM);
    }
    if (j1 >= kmin) break;  // no next panel
    const int jbn = std::min(W, kmin - j1);
    if (look) {
      LA_TRY(trailing(j0, jb, j1, j1 + jbn, 0));
      LA_CUDA(ctx, cudaEventRecord(ctx->ev_fork, ms));
      LA_CUDA(ctx, cudaStreamWaitEvent(ss, ctx->ev_fork, 0));
      b = t.begin(ss);
      LA_TRY(launch_panel(ctx, ss, exact, A, S.d(), ld, m, j1, jbn, h->d_ipiv, &bar_base));
      t.end(ss, b, PH_PANEL);
      LA_CUDA(ctx, cudaEventRecord(ctx->ev_join, ss));
      LA_TRY(trailing(j0, jb, j1 + jbn, n, GEMM_SMEM_WITH_PANEL));
      LA_CUDA(ctx, cudaStreamWaitEvent(ms, ctx->ev_join, 0));
    } else {
      LA_TRY(trailing(j0, jb, j1, n, 0));
      b = t.begin(ms);
      LA_TRY(launch_panel(ctx, ms, exact, A, S.d(), ld, m, j1, jbn, h->d_ipiv, &bar_base));
      t.end(ms, b, PH_PANEL);
    }
  }
  // m < n: the columns right of the last panel got their triangular update above.
  size_t b = t.begin(ms);
  LA_TRY(launch_lu_finish(ctx, h, d_flags));
  t.end(ms, b, PH_OTHER);
  if (t.on) {
    LA_CUDA(ctx, cudaStreamSynchronize(ms));
    t.finish();
  } else {
    for (int i = 0; i < 5; i++) ctx->phase_ms[i] = 0;
  }
  return LA_OK;
}

namespace {

la_status lu_factor(la_ctx ctx, la_lu h) {
  int* d_flags = reinterpret_cast<int*>(ctx->d_small);
  LA_TRY(lu_factor_enqueue(ctx, h, d_flags));
  int* flags = static_cast<int*>(ctx->h_pinned);
  LA_CUDA(ctx, cudaMemcpyAsync(flags, d_flags, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  LA_TRY(la_sync_and_check(ctx, "lu factorization"));
  h->pospivsign = flags[0];
  h->zero_diag = flags[1];
  return LA_OK;
}

la_status lu_alloc(la_ctx ctx, size_t m, size_t n, la_lu* out) {
  if (m == 0 || n == 0) return LA_BADSHAPE;  // Matrix::new asserts (mod.rs:209)
  if (m > (size_t)INT32_MAX / 2 || n > (size_t)INT32_MAX / 2) return LA_UNSUPPORTED;
  la_lu h = new (std::nothrow) la_lu_handle();
  if (!h) return LA_NOMEM;
  h->ctx = ctx;
  h->m = m;
  h->n = n;
  h->ld = pad4(n);
  h->arith = ctx->arith;
  void* p = nullptr;
  la_status s = la_device_alloc(ctx, &p, m * h->ld * sizeof(double));
  if (s != LA_OK) { delete h; return s; }
  h->d_lu = static_cast<double*>(p);
  s = la_device_alloc(ctx, &p, std::min(m, n) * sizeof(int));
  if (s != LA_OK) { la_lu_free(h); return s; }
  h->d_ipiv = static_cast<int*>(p);
  s = la_device_alloc(ctx, &p, m * sizeof(uint64_t));
  if (s != LA_OK) { la_lu_free(h); return s; }
  h->d_piv = static_cast<uint64_t*>(p);
  *out = h;
  return LA_OK;
}

// is_non_singular (lu.rs:174-182) from the factorization's zero flag: a zero
// among U's first min(m,n) diagonal entries returns false first; with m < n the
// reference's index j*n+j leaves its data at j = m, which panics.
la_status lu_non_singular(la_lu h, int* out) {
  if (h->zero_diag) { *out = 0; return LA_OK; }
  if (h->m < h->n) return LA_BADSHAPE;
  *out = 1;
  return LA_OK;
}

// X (m x nrhs, pitch ldx) holds B(piv,:) on entry and the solution on exit
// (lu.rs:256-275; the loops run over the first n rows).
la_status lu_solve_inplace(la_ctx ctx, la_lu h, double* X, size_t ldx, int nrhs) {
  return launch_lu_solve(ctx, h->arith == LA_ARITH_EXACT, h->d_lu, h->ld, X, ldx, (int)h->n,
                         nrhs);
}

la_status check_ctx(la_ctx ctx) {
  if (!ctx) return LA_INVALID;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaSetDevice");
  return LA_OK;
}

// Device solve shared by the host and device entry points: d_b (pitch ldb) ->
// d_x (pitch ldx); both may be unaligned, an aligned work buffer is used.
la_status solve_device_common(la_lu h, const double* d_b, size_t ldb, size_t brows, size_t nrhs,
                              double* d_x, size_t ldx) {
  la_ctx ctx = h->ctx;
  if (brows != h->m) return LA_BADSHAPE;  // lu.rs:240
  if (nrhs == 0) return LA_BADSHAPE;      // Matrix::new asserts cols > 0
  int ns = 0;
  LA_TRY(lu_non_singular(h, &ns));        // lu.rs:241
  if (!ns) return LA_SINGULAR;
  const size_t ldw = pad4(nrhs);
  DevBuf Xw(ctx);
  LA_TRY(Xw.alloc(h->m * ldw * sizeof(double)));
  LA_TRY(launch_permute_rows(ctx, h->d_piv, d_b, ldb, Xw.d(), ldw, (int)h->m, (int)nrhs));
  LA_TRY(lu_solve_inplace(ctx, h, Xw.d(), ldw, (int)nrhs));
  LA_CUDA(ctx, cudaMemcpy2DAsync(d_x, ldx * sizeof(double), Xw.d(), ldw * sizeof(double),
                                 nrhs * sizeof(double), h->m, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
  return LA_OK;
}

la_status gemm_device_common(la_ctx ctx, const double* d_a, size_t lda, const double* d_b,
                             size_t ldb, double* d_c, size_t ldc, size_t m, size_t k, size_t n) {
  const int mode = ctx->arith == LA_ARITH_EXACT ? GM_EXACT_ZERO : GM_FMA_ZERO;
  DevBuf a2(ctx), b2(ctx), c2(ctx);
  const double* A = d_a;
  const double* B = d_b;
  double* C = d_c;
  size_t la = lda, lb = ldb, lc = ldc;
  if (!aligned16(d_a, lda)) {
    la = pad4(k);
    LA_TRY(a2.alloc(m * la * sizeof(double)));
    LA_CUDA(ctx, cudaMemcpy2DAsync(a2.p, la * 8, d_a, lda * 8, k * 8, m, cudaMemcpyDeviceToDevice,
                                   ctx->stream));
    A = a2.d();
  }
  if (!aligned16(d_b, ldb)) {
    lb = pad4(n);
    LA_TRY(b2.alloc(k * lb * sizeof(double)));
    LA_CUDA(ctx, cudaMemcpy2DAsync(b2.p, lb * 8, d_b, ldb * 8, n * 8, k, cudaMemcpyDeviceToDevice,
                                   ctx->stream));
    B = b2.d();
  }
  if (!aligned16(d_c, ldc)) {
    lc = pad4(n);
    LA_TRY(c2.alloc(m * lc * sizeof(double)));
    C = c2.d();
  }
  LA_TRY(launch_gemm(ctx, mode, (int)m, (int)n, (int)k, A, la, B, lb, C, lc));
  if (C != d_c)
    LA_CUDA(ctx, cudaMemcpy2DAsync(d_c, ldc * 8, C, lc * 8, n * 8, m, cudaMemcpyDeviceToDevice,
                                   ctx->stream));
  return LA_OK;
}

la_status fetch(la_ctx ctx, void* host, const void* dev, size_t bytes) {
  LA_CUDA(ctx, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return la_sync_and_check(ctx, "readback");
}

}  // namespace

extern "C" {

la_status la_lu_new(la_ctx ctx, const double* a, size_t m, size_t n, la_lu* out) {
  LA_TRY(check_ctx(ctx));
  if (!a || !out) return LA_INVALID;
  *out = nullptr;
  la_lu h = nullptr;
  LA_TRY(lu_alloc(ctx, m, n, &h));
  la_status s = LA_OK;
  cudaError_t e = cudaMemcpy2DAsync(h->d_lu, h->ld * sizeof(double), a, n * sizeof(double),
                                    n * sizeof(double), m, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) s = la_cuda_fail(ctx, e, "copy A to device");
  if (s == LA_OK) s = lu_factor(ctx, h);
  if (s != LA_OK) { la_lu_free(h); return s; }
  *out = h;
  return LA_OK;
}

la_status la_lu_new_device(la_ctx ctx, const double* d_a, size_t lda, size_t m, size_t n,
                           la_lu* out) {
  LA_TRY(check_ctx(ctx));
  if (!d_a || !out || lda < n) return LA_INVALID;
  *out = nullptr;
  la_lu h = nullptr;
  LA_TRY(lu_alloc(ctx, m, n, &h));
  la_status s = LA_OK;
  cudaError_t e = cudaMemcpy2DAsync(h->d_lu, h->ld * sizeof(double), d_a, lda * sizeof(double),
                                    n * sizeof(double), m, cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) s = la_cuda_fail(ctx, e, "copy A on device");
  if (s == LA_OK) s = lu_factor(ctx, h);
  if (s != LA_OK) { la_lu_free(h); return s; }
  *out = h;
  return LA_OK;
}

void la_lu_free(la_lu h) {
  if (!h) return;
  la_ctx ctx = h->ctx;
  cudaSetDevice(ctx->device);
  la_device_free(ctx, h->d_lu);
  la_device_free(ctx, h->d_lu32);
  la_device_free(ctx, h->d_dinv);
  la_device_free(ctx, h->d_dinvf);
  la_device_free(ctx, h->d_ipiv);
  la_device_free(ctx, h->d_piv);
  delete h;
}

la_status la_lu_shape(la_lu h, size_t* m, size_t* n) {
  if (!h) return LA_INVALID;
  if (m) *m = h->m;
  if (n) *n = h->n;
  return LA_OK;
}

la_status la_lu_is_non_singular(la_lu h, int* out) {
  if (!h || !out) return LA_INVALID;
  return lu_non_singular(h, out);
}

la_status la_lu_det(la_lu h, double* out) {
  if (!h || !out) return LA_INVALID;
  la_ctx ctx = h->ctx;
  LA_TRY(check_ctx(ctx));
  if (h->m != h->n) return LA_BADSHAPE;  // lu.rs:225
  LA_TRY(launch_det(ctx, h->d_lu, h->ld, (int)h->n, h->pospivsign, ctx->d_small + 2));
  double* hp = static_cast<double*>(ctx->h_pinned);
  LA_TRY(fetch(ctx, hp, ctx->d_small + 2, sizeof(double)));
  *out = hp[0];
  return LA_OK;
}

la_status la_lu_get_piv(la_lu h, uint64_t* piv, int* pospivsign) {
  if (!h) return LA_INVALID;
  if (pospivsign) *pospivsign = h->pospivsign;
  if (piv) {
    LA_TRY(check_ctx(h->ctx));
    LA_TRY(fetch(h->ctx, piv, h->d_piv, h->m * sizeof(uint64_t)));
  }
  return LA_OK;
}

static la_status get_unpacked(la_lu h, int which, double* out) {
  if (!h || !out) return LA_INVALID;
  la_ctx ctx = h->ctx;
  LA_TRY(check_ctx(ctx));
  const size_t kmin = std::min(h->m, h->n);
  size_t rows = which == 0 ? h->m : which == 1 ? kmin : h->m;
  size_t cols = which == 0 ? kmin : which == 1 ? h->n : which == 2 ? h->m : h->n;
  DevBuf tmp(ctx);
  LA_TRY(tmp.alloc(rows * cols * sizeof(double)));
  LA_TRY(launch_unpack(ctx, which, h->d_lu, h->ld, (int)h->m, (int)h->n, h->d_piv, tmp.d()));
  return fetch(ctx, out, tmp.p, rows * cols * sizeof(double));
}

la_status la_lu_get_l(la_lu h, double* out) { return get_unpacked(h, 0, out); }
la_status la_lu_get_u(la_lu h, double* out) { return get_unpacked(h, 1, out); }
la_status la_lu_get_p(la_lu h, double* out) { return get_unpacked(h, 2, out); }
la_status la_lu_get_packed(la_lu h, double* out) { return get_unpacked(h, 3, out); }

const double* la_lu_device_data(la_lu h, size_t* ld) {
  if (!h) return nullptr;
  if (ld) *ld = h->ld;
  return h->d_lu;
}

la_status la_lu_solve(la_lu h, const double* b, size_t brows, size_t nrhs, double* x) {
  if (!h || !b || !x) return LA_INVALID;
  la_ctx ctx = h->ctx;
  LA_TRY(check_ctx(ctx));
  if (brows != h->m) return LA_BADSHAPE;
  if (nrhs == 0) return LA_BADSHAPE;
  int ns = 0;
  LA_TRY(lu_non_singular(h, &ns));
  if (!ns) return LA_SINGULAR;
  const size_t ldw = pad4(nrhs);
  DevBuf Bd(ctx), Xw(ctx);
  LA_TRY(Bd.alloc(h->m * nrhs * sizeof(double)));
  LA_TRY(Xw.alloc(h->m * ldw * sizeof(double)));
  LA_CUDA(ctx, cudaMemcpyAsync(Bd.p, b, h->m * nrhs * sizeof(double), cudaMemcpyHostToDevice,
                               ctx->stream));
  LA_TRY(launch_permute_rows(ctx, h->d_piv, Bd.d(), nrhs, Xw.d(), ldw, (int)h->m, (int)nrhs));
  LA_TRY(lu_solve_inplace(ctx, h, Xw.d(), ldw, (int)nrhs));
  LA_CUDA(ctx, cudaMemcpy2DAsync(x, nrhs * sizeof(double), Xw.p, ldw * sizeof(double),
                                 nrhs * sizeof(double), h->m, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  return la_sync_and_check(ctx, "lu solve");
}

la_status la_lu_solve_device(la_lu h, const double* d_b, size_t ldb, size_t brows, size_t nrhs,
                             double* d_x, size_t ldx) {
  if (!h || !d_b || !d_x || ldb < nrhs || ldx < nrhs) return LA_INVALID;
  LA_TRY(check_ctx(h->ctx));
  return solve_device_common(h, d_b, ldb, brows, nrhs, d_x, ldx);
}

la_status la_matrix_det(la_ctx ctx, const double* a, size_t m, size_t n, double* out) {
  if (!a || !out) return LA_INVALID;
  if (m != n) return LA_BADSHAPE;  // mod.rs:1026
  la_lu h = nullptr;
  LA_TRY(la_lu_new(ctx, a, m, n, &h));
  la_status s = la_lu_det(h, out);
  la_lu_free(h);
  return s;
}

la_status la_matrix_solve(la_ctx ctx, const double* a, size_t m, size_t n, const double* b,
                          size_t brows, size_t nrhs, double* x) {
  if (!a || !b || !x) return LA_INVALID;
  la_lu h = nullptr;
  LA_TRY(la_lu_new(ctx, a, m, n, &h));
  la_status s = la_lu_solve(h, b, brows, nrhs, x);
  la_lu_free(h);
  return s;
}

la_status la_matrix_inverse(la_ctx ctx, const double* a, size_t m, size_t n, double* out) {
  if (!a || !out) return LA_INVALID;
  if (m != n) return LA_BADSHAPE;  // mod.rs:1035
  la_lu h = nullptr;
  LA_TRY(la_lu_new(ctx, a, m, n, &h));
  la_status s = LA_OK;
  int ns = 0;
  s = lu_non_singular(h, &ns);
  if (s == LA_OK && !ns) s = LA_SINGULAR;
  if (s == LA_OK) {
    const size_t ldw = pad4(n);
    DevBuf Xw(ctx);
    s = Xw.alloc(n * ldw * sizeof(double));
    if (s == LA_OK) s = launch_identity_permuted(ctx, h->d_piv, Xw.d(), ldw, (int)n);
    if (s == LA_OK) s = lu_solve_inplace(ctx, h, Xw.d(), ldw, (int)n);
    if (s == LA_OK) {
      cudaError_t e = cudaMemcpy2DAsync(out, n * sizeof(double), Xw.p, ldw * sizeof(double),
                                        n * sizeof(double), n, cudaMemcpyDeviceToHost,
                                        ctx->stream);
      if (e != cudaSuccess) s = la_cuda_fail(ctx, e, "copy inverse");
    }
    if (s == LA_OK) s = la_sync_and_check(ctx, "inverse");
  }
  la_lu_free(h);
  return s;
}

la_status la_matrix_is_non_singular(la_ctx ctx, const double* a, size_t m, size_t n, int* out) {
  if (!a || !out) return LA_INVALID;
  if (m != n) return LA_BADSHAPE;  // mod.rs:1045
  la_lu h = nullptr;
  LA_TRY(la_lu_new(ctx, a, m, n, &h));
  la_status s = lu_non_singular(h, out);
  la_lu_free(h);
  return s;
}

la_status la_matrix_mul(la_ctx ctx, const double* a, size_t m, size_t k, const double* b,
                        size_t brows, size_t n, double* c) {
  LA_TRY(check_ctx(ctx));
  if (!a || !b || !c) return LA_INVALID;
  if (m == 0 || k == 0 || brows == 0 || n == 0) return LA_BADSHAPE;
  if (k != brows) return LA_BADSHAPE;  // mod.rs:961
  if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX) return LA_UNSUPPORTED;
  const size_t la = pad4(k), lb = pad4(n), lc = pad4(n);
  DevBuf A(ctx), B(ctx), C(ctx);
  LA_TRY(A.alloc(m * la * sizeof(double)));
  LA_TRY(B.alloc(k * lb * sizeof(double)));
  LA_TRY(C.alloc(m * lc * sizeof(double)));
  LA_CUDA(ctx, cudaMemcpy2DAsync(A.p, la * 8, a, k * 8, k * 8, m, cudaMemcpyHostToDevice,
                                 ctx->stream));
  LA_CUDA(ctx, cudaMemcpy2DAsync(B.p, lb * 8, b, n * 8, n * 8, k, cudaMemcpyHostToDevice,
                                 ctx->stream));
  LA_TRY(gemm_device_common(ctx, A.d(), la, B.d(), lb, C.d(), lc, m, k, n));
  LA_CUDA(ctx, cudaMemcpy2DAsync(c, n * 8, C.p, lc * 8, n * 8, m, cudaMemcpyDeviceToHost,
                                 ctx->stream));
  return la_sync_and_check(ctx, "matrix mul");
}

la_status la_matrix_mmul(la_ctx ctx, const double* a, size_t m, size_t k, const double* b,
                         size_t brows, size_t n, double* dst, size_t dst_rows, size_t dst_cols) {
  if (k != brows) return LA_BADSHAPE;                    // mmatrix.rs:83
  if (dst_rows != m || dst_cols != n) return LA_BADSHAPE;  // mmatrix.rs:84-85
  return la_matrix_mul(ctx, a, m, k, b, brows, n, dst);
}

la_status la_matrix_mul_device(la_ctx ctx, const double* d_a, size_t lda, const double* d_b,
                               size_t ldb, double* d_c, size_t ldc, size_t m, size_t k, size_t n) {
  LA_TRY(check_ctx(ctx));
  if (!d_a || !d_b || !d_c || lda < k || ldb < n || ldc < n) return LA_INVALID;
  if (m == 0 || k == 0 || n == 0) return LA_BADSHAPE;
  if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX) return LA_UNSUPPORTED;
  return gemm_device_common(ctx, d_a, lda, d_b, ldb, d_c, ldc, m, k, n);
}

}  // extern "C"
