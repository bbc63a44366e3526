// Normwise backward error of a computed solution, on the device:
//   eta = max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf)
// The residual is accumulated with error-free transformations (TwoProduct by
// FMA, TwoSum), so its own rounding is far below the eta it measures; this is
// the FP64 check every result of the LU path is reported with (the reference
// has no counterpart).
//
// One warp per row of A: lanes stride along the row (coalesced), each lane keeps
// a compensated sum per right-hand side, the warp combines them, and the
// per-column maxima are merged with an integer atomicMax on the IEEE bits of
// non-negative doubles (their order matches the integers').
#include "la_internal.cuh"

#include <vector>

namespace {

constexpr int RES_MAX_RHS = 16;

__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double bv = s - a;
  double av = s - bv;
  e = (a - av) + (b - bv);
}

__device__ __forceinline__ void atomic_max_nonneg(double* addr, double v) {
  // For v >= 0 (and +inf / NaN bit patterns above them) the unsigned order of
  // the bits is the numeric order.
  atomicMax(reinterpret_cast<unsigned long long*>(addr),
            static_cast<unsigned long long>(__double_as_longlong(v)));
}

template <int R>
__global__ void __launch_bounds__(256)
residual_kernel(const double* __restrict__ A, size_t lda, const double* __restrict__ X, size_t ldx,
                const double* __restrict__ B, size_t ldb, int n, int nrhs, int j0,
                double* __restrict__ out /* [0]=||A||inf, [1+j]=rmax_j, [1+R+j]=xmax_j,
                                            [1+2R+j]=bmax_j */) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = warp; i < n; i += nwarps) {
    double s[R], c[R];
#pragma unroll
    for (int j = 0; j < R; j++) { s[j] = 0.0; c[j] = 0.0; }
    double asum = 0.0;
    const double* arow = A + (size_t)i * lda;
    for (int k = lane; k < n; k += 32) {
      const double a = arow[k];
      asum += fabs(a);
      const double* xr = X + (size_t)k * ldx + j0;
#pragma unroll
      for (int j = 0; j < R; j++) {
        if (j < nrhs) {
          const double x = xr[j];
          const double p = -a * x;
          const double pe = fma(-a, x, -p);
          double t, te;
          two_sum(s[j], p, t, te);
          s[j] = t;
          c[j] += pe + te;
        }
      }
    }
    // Warp reduction of the compensated sums.
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      asum += __shfl_down_sync(0xffffffffu, asum, off);
#pragma unroll
      for (int j = 0; j < R; j++) {
        double os = __shfl_down_sync(0xffffffffu, s[j], off);
        double oc = __shfl_down_sync(0xffffffffu, c[j], off);
        double t, te;
        two_sum(s[j], os, t, te);
        s[j] = t;
        c[j] += oc + te;
      }
    }
    if (lane == 0) {
      atomic_max_nonneg(out, asum);
#pragma unroll
      for (int j = 0; j < R; j++) {
        if (j < nrhs) {
          const double bij = B[(size_t)i * ldb + j0 + j];
          double t, te;
          two_sum(s[j], bij, t, te);
          const double r = fabs(t + (c[j] + te));
          atomic_max_nonneg(out + 1 + j, r);
          atomic_max_nonneg(out + 1 + R + j, fabs(X[(size_t)i * ldx + j0 + j]));
          atomic_max_nonneg(out + 1 + 2 * R + j, fabs(bij));
        }
      }
    }
  }
}

la_status eta_device(la_ctx ctx, const double* A, size_t lda, const double* X, size_t ldx,
                     const double* B, size_t ldb, int n, int nrhs, double* eta) {
  double worst = 0.0;
  const size_t nslots = 1 + 3 * RES_MAX_RHS;
  double* d_out = nullptr;
  LA_TRY(la_device_alloc(ctx, reinterpret_cast<void**>(&d_out), nslots * sizeof(double)));
  std::vector<double> h(nslots);
  la_status st = LA_OK;
  for (int j0 = 0; j0 < nrhs && st == LA_OK; j0 += RES_MAX_RHS) {
    const int cnt = std::min(RES_MAX_RHS, nrhs - j0);
    cudaError_t e = cudaMemsetAsync(d_out, 0, nslots * sizeof(double), ctx->stream);
    if (e != cudaSuccess) { st = la_cuda_fail(ctx, e, "memset eta"); break; }
    const int blocks = std::min((n + 7) / 8, ctx->sm_count * 8);
    residual_kernel<RES_MAX_RHS><<<blocks, 256, 0, ctx->stream>>>(A, lda, X, ldx, B, ldb, n, cnt,
                                                                 j0, d_out);
    ctx->launches++;
    st = la_check_launch(ctx, "residual_kernel");
    if (st != LA_OK) break;
    e = cudaMemcpyAsync(h.data(), d_out, nslots * sizeof(double), cudaMemcpyDeviceToHost,
                        ctx->stream);
    if (e != cudaSuccess) { st = la_cuda_fail(ctx, e, "copy eta"); break; }
    st = la_sync_and_check(ctx, "backward error");
    if (st != LA_OK) break;
    const double anorm = h[0];
    for (int j = 0; j < cnt; j++) {
      const double r = h[1 + j], xm = h[1 + RES_MAX_RHS + j], bm = h[1 + 2 * RES_MAX_RHS + j];
      const double den = anorm * xm + bm;
      const double v = den > 0 ? r / den : (r > 0 ? INFINITY : 0.0);
      if (!(v <= worst)) worst = v;  // keeps NaN
    }
  }
  la_device_free(ctx, d_out);
  if (st == LA_OK) *eta = worst;
  return st;
}

// Backward error of every system of a batch: one CTA per system (grid-stride
// over the systems), warps over its rows, the same compensated residual as
// residual_kernel, right-hand sides in groups of BE_R, the maxima merged in
// shared memory; thread 0 writes the system's eta.
constexpr int BE_R = 4;

__global__ void __launch_bounds__(256)
batch_eta_kernel(const double* __restrict__ A, const double* __restrict__ B,
                 const double* __restrict__ X, const la_batch_system* __restrict__ sys, int count,
                 double* __restrict__ eta_out) {
  __shared__ double s_max[1 + 3 * BE_R];
  __shared__ double s_worst;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int q = blockIdx.x; q < count; q += gridDim.x) {
    const la_batch_system d = sys[q];
    const int n = d.n, nrhs = d.nrhs;
    const double* Ai = A + d.a_offset;
    const double* Bi = B + d.b_offset;
    const double* Xi = X + d.b_offset;
    if (threadIdx.x == 0) s_worst = 0.0;
    for (int j0 = 0; j0 < nrhs; j0 += BE_R) {
      const int cnt = min(BE_R, nrhs - j0);
      if (threadIdx.x < 1 + 3 * BE_R) s_max[threadIdx.x] = 0.0;
      __syncthreads();
      for (int i = warp; i < n; i += nw) {
        double s[BE_R], c[BE_R];
#pragma unroll
        for (int j = 0; j < BE_R; j++) { s[j] = 0.0; c[j] = 0.0; }
        double asum = 0.0;
        const double* arow = Ai + (size_t)i * n;
        for (int k = lane; k < n; k += 32) {
          const double a = arow[k];
          asum += fabs(a);
          const double* xr = Xi + (size_t)k * nrhs + j0;
#pragma unroll
          for (int j = 0; j < BE_R; j++) {
            if (j < cnt) {
              const double x = xr[j];
              const double p = -a * x;
              const double pe = fma(-a, x, -p);
              double t, te;
              two_sum(s[j], p, t, te);
              s[j] = t;
              c[j] += pe + te;
            }
          }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          asum += __shfl_down_sync(0xffffffffu, asum, off);
#pragma unroll
          for (int j = 0; j < BE_R; j++) {
            const double os = __shfl_down_sync(0xffffffffu, s[j], off);
            const double oc = __shfl_down_sync(0xffffffffu, c[j], off);
            double t, te;
            two_sum(s[j], os, t, te);
            s[j] = t;
            c[j] += oc + te;
          }
        }
        if (lane == 0) {
          atomic_max_nonneg(s_max, asum);
#pragma unroll
          for (int j = 0; j < BE_R; j++) {
            if (j < cnt) {
              const double bij = Bi[(size_t)i * nrhs + j0 + j];
              double t, te;
              two_sum(s[j], bij, t, te);
              atomic_max_nonneg(s_max + 1 + j, fabs(t + (c[j] + te)));
              atomic_max_nonneg(s_max + 1 + BE_R + j, fabs(Xi[(size_t)i * nrhs + j0 + j]));
              atomic_max_nonneg(s_max + 1 + 2 * BE_R + j, fabs(bij));
            }
          }
        }
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double worst = s_worst;
        for (int j = 0; j < cnt; j++) {
          const double r = s_max[1 + j];
          const double den = s_max[0] * s_max[1 + BE_R + j] + s_max[1 + 2 * BE_R + j];
          const double v = den > 0 ? r / den : (r > 0 ? INFINITY : 0.0);
          if (!(v <= worst)) worst = v;  // keeps NaN
        }
        s_worst = worst;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) eta_out[q] = s_worst;
    __syncthreads();
  }
}

}  // namespace

extern "C" {

la_status la_batch_backward_error_device(la_ctx ctx, const double* d_a, const double* d_b,
                                         const double* d_x, const la_batch_system* systems,
                                         int count, double* d_eta, double* max_eta) {
  if (!ctx || !d_a || !d_b || !d_x || !systems || !d_eta || count < 0) return LA_INVALID;
  for (int i = 0; i < count; i++)
    if (systems[i].n < 1 || systems[i].nrhs < 1) return LA_BADSHAPE;
  if (count == 0) {
    if (max_eta) *max_eta = 0.0;
    return LA_OK;
  }
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  la_batch_system* d_sys = nullptr;
  LA_TRY(la_device_alloc(ctx, reinterpret_cast<void**>(&d_sys),
                         (size_t)count * sizeof(la_batch_system)));
  la_status st = LA_OK;
  cudaError_t e = cudaMemcpyAsync(d_sys, systems, (size_t)count * sizeof(la_batch_system),
                                  cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) st = la_cuda_fail(ctx, e, "copy batch descriptors");
  if (st == LA_OK) {
    const int grid = std::min(count, ctx->sm_count * 8);
    batch_eta_kernel<<<grid, 256, 0, ctx->stream>>>(d_a, d_b, d_x, d_sys, count, d_eta);
    ctx->launches++;
    st = la_check_launch(ctx, "batch_eta_kernel");
  }
  if (st == LA_OK && max_eta) {
    std::vector<double> h(count);
    e = cudaMemcpyAsync(h.data(), d_eta, (size_t)count * sizeof(double), cudaMemcpyDeviceToHost,
                        ctx->stream);
    if (e != cudaSuccess) st = la_cuda_fail(ctx, e, "copy batch eta");
    if (st == LA_OK) st = la_sync_and_check(ctx, "batch backward error");
    if (st == LA_OK) {
      double worst = 0.0;
      for (double v : h)
        if (!(v <= worst)) worst = v;  // keeps NaN
      *max_eta = worst;
    }
  } else if (st == LA_OK) {
    st = la_sync_and_check(ctx, "batch backward error");
  }
  la_device_free(ctx, d_sys);
  return st;
}

la_status la_backward_error_device(la_ctx ctx, const double* d_a, size_t lda, const double* d_x,
                                   size_t ldx, const double* d_b, size_t ldb, size_t n,
                                   size_t nrhs, double* eta) {
  if (!ctx || !d_a || !d_x || !d_b || !eta || lda < n || ldx < nrhs || ldb < nrhs)
    return LA_INVALID;
  if (n == 0 || nrhs == 0) return LA_BADSHAPE;
  if (n > INT32_MAX || nrhs > INT32_MAX) return LA_UNSUPPORTED;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  return eta_device(ctx, d_a, lda, d_x, ldx, d_b, ldb, (int)n, (int)nrhs, eta);
}

la_status la_backward_error(la_ctx ctx, const double* a, const double* x, const double* b,
                            size_t n, size_t nrhs, double* eta) {
  if (!ctx || !a || !x || !b || !eta) return LA_INVALID;
  if (n == 0 || nrhs == 0) return LA_BADSHAPE;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  double *dA = nullptr, *dX = nullptr, *dB = nullptr;
  la_status st = la_device_alloc(ctx, reinterpret_cast<void**>(&dA), n * n * sizeof(double));
  if (st == LA_OK) st = la_device_alloc(ctx, reinterpret_cast<void**>(&dX), n * nrhs * 8);
  if (st == LA_OK) st = la_device_alloc(ctx, reinterpret_cast<void**>(&dB), n * nrhs * 8);
  if (st == LA_OK) {
    cudaError_t e = cudaMemcpyAsync(dA, a, n * n * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dX, x, n * nrhs * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dB, b, n * nrhs * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) st = la_cuda_fail(ctx, e, "copy for backward error");
  }
  if (st == LA_OK) st = eta_device(ctx, dA, n, dX, nrhs, dB, nrhs, (int)n, (int)nrhs, eta);
  la_device_free(ctx, dA);
  la_device_free(ctx, dX);
  la_device_free(ctx, dB);
  cudaStreamSynchronize(ctx->stream);
  return st;
}

}  // extern "C"
