// GMRES-based iterative refinement (Carson and Higham's GMRES-IR) for the
// mixed-precision LU, used when plain refinement stalls on an ill-conditioned
// matrix (kappa(A) * u_factor >= 1).
//
// Each refinement step solves A d = r by GMRES on the left-preconditioned
// system M^-1 A d = M^-1 r, M = P^T L U from the low-precision factorization:
//   matvec      w = M^-1 (A v): A v in FP64 (one warp per row), then the
//               wavefront triangular solves with the FP32 factors at FP64
//   Arnoldi     classical Gram-Schmidt applied twice (CGS2) in FP64
//   least squares Givens rotations on the small Hessenberg matrix (host)
// then x += d (FP64) and r = b - A x (FP64). The preconditioner is applied at
// working precision (FP64 vectors over the FP32 factors): applied in FP32 its
// rounding, amplified by kappa(U), breaks the Arnoldi relation for
// ill-conditioned matrices.
#include "la_internal.cuh"

namespace {

int gridn(la_ctx ctx, size_t total) {
  size_t g = (total + 255) / 256;
  return (int)std::max<size_t>(1, std::min(g, (size_t)ctx->sm_count * 8));
}

// w = A v (FP64), one warp per row.
__global__ void gemv_kernel(const double* __restrict__ A, size_t lda, const double* __restrict__ v,
                            double* __restrict__ w, int n) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = warp; i < n; i += nw) {
    const double* a = A + (size_t)i * lda;
    double s = 0.0;
    for (int k = lane; k < n; k += 32) s = fma(a[k], v[k], s);
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) w[i] = s;
  }
}

// z[i] = v[piv[i]]
__global__ void perm_kernel(const uint64_t* __restrict__ piv, const double* __restrict__ v,
                            double* __restrict__ z, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    z[i] = v[piv[i]];
}

// h[i] += sum over this block's chunk of V_i . w for i < k (h zeroed before).
__global__ void multi_dot_kernel(const double* __restrict__ V, size_t ldv, int k,
                                 const double* __restrict__ w, int n, double* h) {
  __shared__ double part[32][33];
  for (int i0 = 0; i0 < k; i0 += 32) {
    const int kk = min(32, k - i0);
    double s[32];
#pragma unroll
    for (int q = 0; q < 32; q++) s[q] = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
      const double wt = w[t];
#pragma unroll
      for (int q = 0; q < 32; q++)
        if (q < kk) s[q] = fma(V[(size_t)(i0 + q) * ldv + t], wt, s[q]);
    }
#pragma unroll
    for (int q = 0; q < 32; q++)
      for (int off = 16; off > 0; off >>= 1) s[q] += __shfl_down_sync(0xffffffffu, s[q], off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 32; q++) part[warp][q] = s[q];
    __syncthreads();
    if (threadIdx.x < kk) {
      double t = 0.0;
      for (int w2 = 0; w2 < (int)(blockDim.x >> 5); w2++) t += part[w2][threadIdx.x];
      atomicAdd(h + i0 + threadIdx.x, t);
    }
    __syncthreads();
  }
}

// w -= sum_{i<k} h[i] V_i
__global__ void multi_axpy_kernel(const double* __restrict__ V, size_t ldv, int k,
                                  const double* __restrict__ h, double* __restrict__ w, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s = w[t];
    for (int i = 0; i < k; i++) s = fma(-h[i], V[(size_t)i * ldv + t], s);
    w[t] = s;
  }
}

// dst = src * a (a on the host)
__global__ void scal_copy_kernel(const double* __restrict__ src, double a, double* __restrict__ dst,
                                 int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    dst[t] = src[t] * a;
}

// x[:, col] += sum_i y[i] V_i  (y on the device)
__global__ void update_col_kernel(const double* __restrict__ V, size_t ldv, int k,
                                  const double* __restrict__ y, double* X, size_t ldx, int col,
                                  int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < k; i++) s = fma(y[i], V[(size_t)i * ldv + t], s);
    X[(size_t)t * ldx + col] += s;
  }
}

__global__ void copy_col_kernel(const double* __restrict__ R, size_t ldr, int col,
                                double* __restrict__ out, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    out[t] = R[(size_t)t * ldr + col];
}

struct Work {
  la_ctx ctx;
  std::vector<void*> ptrs;
  explicit Work(la_ctx c) : ctx(c) {}
  ~Work() {
    for (void* p : ptrs) la_device_free(ctx, p);
  }
  template <typename T>
  la_status get(T** out, size_t count) {
    void* p = nullptr;
    LA_TRY(la_device_alloc(ctx, &p, count * sizeof(T)));
    ptrs.push_back(p);
    *out = static_cast<T*>(p);
    return LA_OK;
  }
};

}  // namespace

// z = M^-1 v with the FP32 factors of h, at FP64 (v, z length n; v != z).
static la_status precond(la_ctx ctx, la_lu h, const double* v, double* z, int* sync) {
  const int n = (int)h->n;
  cudaStream_t st = ctx->stream;
  perm_kernel<<<gridn(ctx, n), 256, 0, st>>>(h->d_piv, v, z, n);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "permute"));
  return launch_trsv_wave_f32(ctx, h->d_lu32, h->ld32, h->d_dinv, z, 1, n, 1, sync);
}

// One GMRES solve of A d = r (column `col` of R), adding d to column `col`
// of X. Returns the number of Arnoldi steps taken.
la_status gmres_correction(la_ctx ctx, la_lu h, const double* R, size_t ldr, int col, double* X,
                           size_t ldx, int m, double tau, int* steps) {
  const int n = (int)h->n;
  cudaStream_t st = ctx->stream;
  Work wk(ctx);
  double *V, *w, *z, *hd;
  int* sync;
  const size_t ldv = (size_t)n;
  LA_TRY(wk.get(&V, (size_t)(m + 1) * ldv));
  LA_TRY(wk.get(&w, n));
  LA_TRY(wk.get(&z, n));
  LA_TRY(wk.get(&hd, 64 + 2 * (size_t)m));
  LA_TRY(wk.get(&sync, 2 * ((n + 63) / 64) + 2));
  double* hh = static_cast<double*>(ctx->h_pinned);  // 4 KB staging: up to 512 doubles

  // z0 = M^-1 r
  copy_col_kernel<<<gridn(ctx, n), 256, 0, st>>>(R, ldr, col, w, n);
  ctx->launches++;
  LA_TRY(precond(ctx, h, w, z, sync));
  LA_CUDA(ctx, cudaMemsetAsync(hd, 0, sizeof(double), st));
  multi_dot_kernel<<<gridn(ctx, n), 256, 0, st>>>(z, ldv, 1, z, n, hd);
  ctx->launches++;
  LA_CUDA(ctx, cudaMemcpyAsync(hh, hd, sizeof(double), cudaMemcpyDeviceToHost, st));
  LA_TRY(la_sync_and_check(ctx, "gmres start"));
  const double beta = std::sqrt(hh[0]);
  *steps = 0;
  if (!(beta > 0.0) || !std::isfinite(beta)) return LA_OK;
  scal_copy_kernel<<<gridn(ctx, n), 256, 0, st>>>(z, 1.0 / beta, V, n);
  ctx->launches++;

  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0);
  g[0] = beta;
  int k = 0;
  for (; k < m; k++) {
    // w = M^-1 A v_k
    gemv_kernel<<<std::min((n + 7) / 8, ctx->sm_count * 8), 256, 0, st>>>(
        h->d_lu, h->ld, V + (size_t)k * ldv, z, n);
    ctx->launches++;
    LA_TRY(precond(ctx, h, z, w, sync));
    // CGS2: two passes of h = V^T w, w -= V h
    std::vector<double> hcol(k + 2, 0.0);
    for (int pass = 0; pass < 2; pass++) {
      LA_CUDA(ctx, cudaMemsetAsync(hd, 0, (k + 1) * sizeof(double), st));
      multi_dot_kernel<<<gridn(ctx, n), 256, 0, st>>>(V, ldv, k + 1, w, n, hd);
      multi_axpy_kernel<<<gridn(ctx, n), 256, 0, st>>>(V, ldv, k + 1, hd, w, n);
      ctx->launches += 2;
      LA_CUDA(ctx, cudaMemcpyAsync(hh, hd, (k + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
      LA_TRY(la_sync_and_check(ctx, "gmres cgs"));
      for (int i = 0; i <= k; i++) hcol[i] += hh[i];
    }
    LA_CUDA(ctx, cudaMemsetAsync(hd, 0, sizeof(double), st));
    multi_dot_kernel<<<gridn(ctx, n), 256, 0, st>>>(w, ldv, 1, w, n, hd);
    ctx->launches++;
    LA_CUDA(ctx, cudaMemcpyAsync(hh, hd, sizeof(double), cudaMemcpyDeviceToHost, st));
    LA_TRY(la_sync_and_check(ctx, "gmres norm"));
    hcol[k + 1] = std::sqrt(hh[0]);
    if (hcol[k + 1] > 0.0 && std::isfinite(hcol[k + 1])) {
      scal_copy_kernel<<<gridn(ctx, n), 256, 0, st>>>(w, 1.0 / hcol[k + 1],
                                                      V + (size_t)(k + 1) * ldv, n);
      ctx->launches++;
    }
    // Givens rotations of the new Hessenberg column
    for (int i = 0; i < k; i++) {
      const double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
      hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
      hcol[i] = t;
    }
    const double rr = std::hypot(hcol[k], hcol[k + 1]);
    cs[k] = rr > 0 ? hcol[k] / rr : 1.0;
    sn[k] = rr > 0 ? hcol[k + 1] / rr : 0.0;
    hcol[k] = rr;
    hcol[k + 1] = 0.0;
    g[k + 1] = -sn[k] * g[k];
    g[k] = cs[k] * g[k];
    for (int i = 0; i <= k; i++) H[(size_t)i * m + k] = hcol[i];
    if (std::fabs(g[k + 1]) <= tau * beta || !(rr > 0.0)) { k++; break; }
  }
  // y = H(0:k,0:k)^-1 g(0:k); d = V y
  std::vector<double> y(k, 0.0);
  for (int i = k - 1; i >= 0; i--) {
    double s = g[i];
    for (int j = i + 1; j < k; j++) s -= H[(size_t)i * m + j] * y[j];
    y[i] = H[(size_t)i * m + i] != 0.0 ? s / H[(size_t)i * m + i] : 0.0;
  }
  for (int i = 0; i < k; i++) hh[i] = y[i];
  LA_CUDA(ctx, cudaMemcpyAsync(hd, hh, k * sizeof(double), cudaMemcpyHostToDevice, st));
  update_col_kernel<<<gridn(ctx, n), 256, 0, st>>>(V, ldv, k, hd, X, ldx, col, n);
  ctx->launches++;
  LA_TRY(la_sync_and_check(ctx, "gmres update"));
  *steps = k;
  return LA_OK;
}
