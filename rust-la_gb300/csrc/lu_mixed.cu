// Mixed-precision LU with FP64 iterative refinement (not in the reference; it
// replaces LUDecomposition::new + solve, lu.rs:104-278, for well- to
// ill-conditioned systems at a fraction of the FP64 cost).
//
// Factorization of an FP32 copy of A, two-level blocked right-looking:
//   outer panels of width WO = 256, each factored by the FP32 form of the
//   plain path with inner width 32 (panel on one thread-block cluster,
//   panel_cluster.cu, or the cooperative kernel; row swaps, row-panel
//   triangular update, FP32 SIMT updates);
//   outer row-panel triangular update U12 = L11^-1 A12 in FP32;
//   trailing update A22 -= L21 * U12 on the tensor cores (gemm_tc.cu) with
//   BF16, FP16, split FP8 e4m3 or split FP16 operands and FP32 accumulation,
//   or in FP32 SIMT (LA_PREC_FP32). FP16 operands use a per-panel power-of-two
//   scale of U12 (L's entries are bounded by 1 under partial pivoting); the
//   split formats scale L21 and U12 by powers of two and store each value as a
//   high and a low part; the scales are undone in the epilogue.
// Solve: x0 = 0, r = b; repeat d = LU32 \ (r scaled to unit max per column),
// x += d (FP64), r = b - A x in FP64 (A kept in FP64), until the normwise
// backward error max_j ||r_j|| / (||A|| ||x_j|| + ||b_j||) <= tol or the
// refinement stalls.
#include <cuda_fp8.h>

#include "la_internal.cuh"

namespace {

constexpr int WO = 256;  // outer panel width (K of the tensor-core update)
constexpr int WI = 32;   // inner panel width (the cluster panel kernel's width)

size_t pad8(size_t x) { return (x + 7) & ~size_t(7); }

__global__ void f64_to_f32_kernel(const double* __restrict__ src, size_t lds, float* __restrict__ dst,
                                  size_t ldd, int rows, int cols) {
  size_t total = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(i / cols), c = (int)(i % cols);
    dst[(size_t)r * ldd + c] = (float)src[(size_t)r * lds + c];
  }
}

template <int FMT>
__device__ __forceinline__ uint16_t to16(float v) {
  if (FMT == LA_LOWP_BF16) {
    __nv_bfloat16 h = __float2bfloat16_rn(v);
    return *reinterpret_cast<uint16_t*>(&h);
  } else {
    __half h = __float2half_rn(v);
    return *reinterpret_cast<uint16_t*>(&h);
  }
}

// L21 (rows x k, pitch lds) -> 16-bit K-major (pitch ldd).
template <int FMT>
__global__ void pack_l_kernel(const float* __restrict__ src, size_t lds, uint16_t* __restrict__ dst,
                              size_t ldd, int rows, int k) {
  la_pdl_wait();
  la_pdl_trigger();
  size_t total = (size_t)rows * ldd;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(i / ldd), c = (int)(i % ldd);
    dst[i] = c < k ? to16<FMT>(src[(size_t)r * lds + c]) : (uint16_t)0;
  }
}

__device__ __forceinline__ void atomic_max_nonneg_f(float* a, float v) {
  atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}

// max |U12| for the FP16 scale (stat[0] must start at 0).
__global__ void absmax_kernel(const float* __restrict__ src, size_t lds, int rows, int cols,
                              float* stat) {
  la_pdl_wait();
  la_pdl_trigger();
  float m = 0.f;
  size_t total = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(i / cols), c = (int)(i % cols);
    float v = fabsf(src[(size_t)r * lds + c]);
    if (v > m) m = v;  // NaN never raises the max
  }
  for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg_f(stat, m);
}

// U12 (k x cols, pitch lds) -> U^T 16-bit K-major (cols x ldd), times scale;
// stat[1] receives alpha = 1/scale. 32x32 tiles through shared memory.
template <int FMT>
__global__ void pack_ut_kernel(const float* __restrict__ src, size_t lds, uint16_t* __restrict__ dst,
                               size_t ldd, int k, int cols, float* stat) {
  la_pdl_wait();
  la_pdl_trigger();
  __shared__ float t[32][33];
  float scale = 1.f;
  if (FMT == LA_LOWP_FP16) {
    // Largest magnitude to about 2^14: far from FP16 overflow, and products
    // accumulate in FP32.
    float mx = stat[0];
    int e = 0;
    if (mx > 0.f && mx < INFINITY) {
      frexpf(mx, &e);
      scale = ldexpf(1.f, 14 - e);
    }
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    stat[1] = 1.f / scale;
  const int c0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int kk = k0 + i, cc = c0 + threadIdx.x;
    t[i][threadIdx.x] = (kk < k && cc < cols) ? src[(size_t)kk * lds + cc] * scale : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int cc = c0 + i, kk = k0 + threadIdx.x;
    if (cc < cols && kk < (int)ldd) dst[(size_t)cc * ldd + kk] = to16<FMT>(t[threadIdx.x][i]);
  }
}

__global__ void set_alpha_one(float* stat) {
  la_pdl_wait();
  la_pdl_trigger();
  stat[0] = 0.f;
  stat[1] = 1.f;
}

// Split storage: v (already scaled) ~ hi + lo with hi = rn(v), lo = rn(v - hi)
// in the storage format (FP8 e4m3 saturating at its largest finite value, or
// FP16).
struct SplitE4M3 {
  using T = uint8_t;
  static constexpr int L_EXP = 8;  // |l| <= 1 -> |l| * 2^8 <= 256 < 448 (e4m3 max)
  static constexpr int U_EXP = 8;  // max |U12| scaled just below 2^8
  static __device__ __forceinline__ void split(float v, T& hi, T& lo) {
    const __nv_fp8_e4m3 h(v);
    const __nv_fp8_e4m3 l(v - static_cast<float>(h));
    hi = h.__x;
    lo = l.__x;
  }
};
struct SplitF16 {
  using T = uint16_t;
  static constexpr int L_EXP = 12;  // products of scaled parts stay far inside FP32
  static constexpr int U_EXP = 14;  // max |U12| scaled just below 2^14 (FP16 max 65504)
  static __device__ __forceinline__ void split(float v, T& hi, T& lo) {
    const __half h = __float2half_rn(v);
    const __half l = __float2half_rn(v - __half2float(h));
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(l);
  }
};

// L21 (rows x k FP32, pitch lds) * 2^L_EXP -> split rows of ldd elements:
// high parts in columns [0, k), low parts in [ldd / 2, ldd / 2 + k), zeros
// elsewhere.
template <typename SP>
__global__ void pack_l_split_kernel(const float* __restrict__ src, size_t lds,
                                    typename SP::T* __restrict__ dst, size_t ldd, int rows, int k) {
  la_pdl_wait();
  la_pdl_trigger();
  const size_t half = ldd / 2;
  const float sl = ldexpf(1.f, SP::L_EXP);
  size_t total = (size_t)rows * half;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / half), c = (int)(i % half);
    typename SP::T hi = 0, lo = 0;
    if (c < k) SP::split(src[(size_t)r * lds + c] * sl, hi, lo);
    dst[(size_t)r * ldd + c] = hi;
    dst[(size_t)r * ldd + half + c] = lo;
  }
}

// U12 (k x cols, pitch lds) -> U^T split (cols rows of ldd elements, as
// pack_l_split_kernel) times a power of two that takes max |U12| (stat[0])
// just below 2^U_EXP; stat[1] receives alpha = 1 / (2^L_EXP * scale). 32x32
// tiles through shared memory.
template <typename SP>
__global__ void pack_ut_split_kernel(const float* __restrict__ src, size_t lds,
                                     typename SP::T* __restrict__ dst, size_t ldd, int k, int cols,
                                     float* stat) {
  la_pdl_wait();
  la_pdl_trigger();
  __shared__ float t[32][33];
  float scale = 1.f;
  const float mx = stat[0];
  int e = 0;
  if (mx > 0.f && mx < INFINITY) {
    frexpf(mx, &e);  // mx = f 2^e, 0.5 <= f < 1
    scale = ldexpf(1.f, SP::U_EXP - e);
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
    stat[1] = 1.f / (ldexpf(1.f, SP::L_EXP) * scale);
  const size_t half = ldd / 2;
  const int c0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int kk = k0 + i, cc = c0 + threadIdx.x;
    t[i][threadIdx.x] = (kk < k && cc < cols) ? src[(size_t)kk * lds + cc] * scale : 0.f;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int cc = c0 + i, kk = k0 + threadIdx.x;
    if (cc < cols && kk < (int)half) {
      typename SP::T hi, lo;
      SP::split(t[threadIdx.x][i], hi, lo);
      dst[(size_t)cc * ldd + kk] = hi;
      dst[(size_t)cc * ldd + half + kk] = lo;
    }
  }
}

// r = b - A x in FP64 for nrhs <= R: the CTA stages 256-row chunks of X in
// shared memory and each of its 8 warps handles RPW rows (lanes stride along
// the row with FMA, then a warp tree); also the per-column maxima of |r|.
template <int R>
__global__ void __launch_bounds__(256)
residual_f64_kernel(const double* __restrict__ A, size_t lda, const double* __restrict__ X,
                    size_t ldx, const double* __restrict__ B, size_t ldb, double* __restrict__ Rout,
                    size_t ldr, int n, int nrhs, double* colmax) {
  constexpr int RPW = R >= 4 ? 1 : 4 / R;
  constexpr int KC = 256;
  __shared__ double xs[KC][R];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = (blockIdx.x * 8 + warp) * RPW;
  double s[RPW][R];
#pragma unroll
  for (int q = 0; q < RPW; q++)
#pragma unroll
    for (int j = 0; j < R; j++) s[q][j] = 0.0;
  for (int k0 = 0; k0 < n; k0 += KC) {
    for (int idx = threadIdx.x; idx < KC * R; idx += 256) {
      const int k = idx / R, j = idx % R;
      xs[k][j] = (k0 + k < n && j < nrhs) ? X[(size_t)(k0 + k) * ldx + j] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < RPW; q++) {
      const int row = row0 + q;
      if (row < n) {
        const double* arow = A + (size_t)row * lda + k0;
        for (int t = lane; t < KC && k0 + t < n; t += 32) {
          const double a = arow[t];
#pragma unroll
          for (int j = 0; j < R; j++) s[q][j] = fma(a, xs[t][j], s[q][j]);
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < RPW; q++)
#pragma unroll
    for (int j = 0; j < R; j++)
      for (int off = 16; off > 0; off >>= 1) s[q][j] += __shfl_down_sync(0xffffffffu, s[q][j], off);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < RPW; q++) {
      const int row = row0 + q;
      if (row >= n) continue;
#pragma unroll
      for (int j = 0; j < R; j++) {
        if (j < nrhs) {
          const double r = B[(size_t)row * ldb + j] - s[q][j];
          Rout[(size_t)row * ldr + j] = r;
          atomicMax(reinterpret_cast<unsigned long long*>(colmax + j),
                    (unsigned long long)__double_as_longlong(fabs(r)));
        }
      }
    }
  }
}

template <int R>
void launch_residual_r(int n, cudaStream_t st, const double* A, size_t lda, const double* X,
                       size_t ldx, const double* B, size_t ldb, double* Rout, size_t ldr, int nrhs,
                       double* colmax) {
  constexpr int ROWS = 8 * (R >= 4 ? 1 : 4 / R);
  residual_f64_kernel<R><<<(n + ROWS - 1) / ROWS, 256, 0, st>>>(A, lda, X, ldx, B, ldb, Rout, ldr,
                                                                n, nrhs, colmax);
}

void launch_residual(int n, int nrhs, cudaStream_t st, const double* A, size_t lda, const double* X,
                     size_t ldx, const double* B, size_t ldb, double* Rout, size_t ldr,
                     double* colmax) {
  if (nrhs <= 1) launch_residual_r<1>(n, st, A, lda, X, ldx, B, ldb, Rout, ldr, nrhs, colmax);
  else if (nrhs <= 2) launch_residual_r<2>(n, st, A, lda, X, ldx, B, ldb, Rout, ldr, nrhs, colmax);
  else if (nrhs <= 4) launch_residual_r<4>(n, st, A, lda, X, ldx, B, ldb, Rout, ldr, nrhs, colmax);
  else if (nrhs <= 8) launch_residual_r<8>(n, st, A, lda, X, ldx, B, ldb, Rout, ldr, nrhs, colmax);
  else launch_residual_r<16>(n, st, A, lda, X, ldx, B, ldb, Rout, ldr, nrhs, colmax);
}

// Column maxima of |M| (rows x cols) into out[0..cols) (non-negative IEEE bits).
__global__ void colmax_kernel(const double* __restrict__ M, size_t ld, int rows, int cols,
                              double* out) {
  size_t total = (size_t)rows * cols;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(i / cols), c = (int)(i % cols);
    double v = fabs(M[(size_t)r * ld + c]);
    atomicMax(reinterpret_cast<unsigned long long*>(out + c),
              (unsigned long long)__double_as_longlong(v));
  }
}

// ||A||_inf: max row sum of |a_ij|.
__global__ void rownorm_kernel(const double* __restrict__ A, size_t lda, int n, double* out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int i = warp; i < n; i += nwarps) {
    double s = 0.0;
    for (int k = lane; k < n; k += 32) s += fabs(A[(size_t)i * lda + k]);
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0)
      atomicMax(reinterpret_cast<unsigned long long*>(out),
                (unsigned long long)__double_as_longlong(s));
  }
}

// w = r(piv,:) / rscale_j in FP32, the right-hand side of a correction solve.
__global__ void scale_permute_kernel(const uint64_t* __restrict__ piv, const double* __restrict__ R,
                                     size_t ldr, const double* __restrict__ rscale,
                                     float* __restrict__ W, size_t ldw, int n, int nrhs) {
  size_t total = (size_t)n * nrhs;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(i / nrhs), c = (int)(i % nrhs);
    const double s = rscale[c];
    const double v = R[(size_t)piv[r] * ldr + c];
    W[(size_t)r * ldw + c] = s > 0 ? (float)(v / s) : 0.f;
  }
}

// x += d * rscale_j (FP64 update of the solution).
__global__ void update_x_kernel(double* __restrict__ X, size_t ldx, const float* __restrict__ D,
                                size_t ldd, const double* __restrict__ rscale, int n, int nrhs) {
  size_t total = (size_t)n * nrhs;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(i / nrhs), c = (int)(i % nrhs);
    X[(size_t)r * ldx + c] += (double)D[(size_t)r * ldd + c] * rscale[c];
  }
}

int grid_for(la_ctx ctx, size_t total) {
  size_t g = (total + 255) / 256;
  return (int)std::max<size_t>(1, std::min(g, (size_t)ctx->sm_count * 8));
}

struct Buf {
  la_ctx ctx;
  void* p = nullptr;
  explicit Buf(la_ctx c) : ctx(c) {}
  ~Buf() { la_device_free(ctx, p); }
  la_status alloc(size_t bytes) { return la_device_alloc(ctx, &p, bytes); }
  template <typename T> T* as() { return static_cast<T*>(p); }
};

}  // namespace

la_status gmres_correction(la_ctx ctx, la_lu h, const double* R, size_t ldr, int col, double* X,
                           size_t ldx, int m, double tau, int* steps);

namespace {

// Inverted diagonal blocks for the wavefront triangular solves (once per handle).
la_status ensure_dinv(la_ctx ctx, la_lu h) {
  const size_t nb = (h->n + 63) / 64;
  void* p = nullptr;
  if (!h->d_dinvf) {
    LA_TRY(la_device_alloc(ctx, &p, nb * 2 * 64 * 64 * sizeof(float)));
    h->d_dinvf = static_cast<float*>(p);
    LA_TRY(launch_invert_diag_f32f(ctx, h->d_lu32, h->ld32, (int)h->n, h->d_dinvf));
  }
  if (!h->d_dinv) {
    LA_TRY(la_device_alloc(ctx, &p, nb * 2 * 64 * 64 * sizeof(double)));
    h->d_dinv = static_cast<double*>(p);
    LA_TRY(launch_invert_diag_f32(ctx, h->d_lu32, h->ld32, (int)h->n, h->d_dinv));
  }
  return LA_OK;
}

// Factors h->d_lu32 (n x n, pitch ld32) in place; pivots into h->d_ipiv.
//
// Schedule with lookahead (outer panel P = [a, b), next Q = [b, c)):
//   after P's inner panels: P's row swaps on the columns >= b (deferred, see
//   below); U12 = L11^-1 A12 for Q's columns; A22 -= L21 U12 on Q's columns;
//   then Q's inner panels start on the high-priority side stream while the
//   main stream finishes U12 and A22 -= L21 U12 on the columns >= c. The two
//   touch disjoint data: Q's panels read and write rows >= b of columns < c
//   (their row swaps are limited to those columns), the rest of the update
//   writes columns >= c and reads L21 and U12 through packed copies. Q's swaps
//   reach the columns >= c after the join, and the update of those columns
//   saw the rows in the order before Q's swaps, consistently with its packed
//   L21. Without lookahead the same steps run on one stream.
la_status mixed_factor(la_ctx ctx, la_lu h, int prec) {
  const int m = (int)h->m, n = (int)h->n;
  const int kmin = std::min(m, n);
  float* A = h->d_lu32;
  const size_t ld = h->ld32;
  cudaStream_t ms = ctx->stream;
  const bool look = ctx->lookahead != 0 && ctx->side_stream != nullptr;
  cudaStream_t ss = look ? ctx->side_stream : ms;
  LA_CUDA(ctx, cudaMemsetAsync(ctx->d_bar, 0, sizeof(unsigned), ms));
  unsigned bar_base = 0;
  Buf lh(ctx), uh(ctx), stat(ctx);
  const size_t ldk = pad8(WO);
  const size_t ldks = 2 * WO;  // split rows: high parts, then low parts from column WO
  if (prec == LA_PREC_FP8) {
    LA_TRY(lh.alloc((size_t)m * ldks + 256));
    LA_TRY(uh.alloc((size_t)n * ldks + 256));
  } else if (prec == LA_PREC_FP16X3) {
    LA_TRY(lh.alloc((size_t)m * ldks * 2 + 256));
    LA_TRY(uh.alloc((size_t)n * ldks * 2 + 256));
  } else if (prec != LA_PREC_FP32) {
    LA_TRY(lh.alloc((size_t)m * ldk * 2 + 256));
    LA_TRY(uh.alloc((size_t)n * ldk * 2 + 256));
  } else {
    LA_TRY(lh.alloc((size_t)m * ldk * 4 + 256));  // FP32 copy of L21
  }
  LA_TRY(stat.alloc(256));
  float* d_stat = stat.as<float>();
  // [0] max |U12|, [1] alpha of the current update
  LA_CUDA(ctx, cudaMemsetAsync(d_stat, 0, 256, ms));

  // Inner panels of the outer panel [j0, j1o) on stream s; row swaps on the
  // columns < climit only.
  auto inner = [&](int j0, int j1o, int climit, cudaStream_t s) -> la_status {
    cudaStream_t saved = ctx->stream;
    ctx->stream = s;
    // panel, row swaps, triangular solve and rank-32 update follow one
    // another on s: each may be scheduled while the one before it finishes
    ctx->pdl_now = ctx->pdl != 0;
    la_status st = LA_OK;
    for (int i0 = j0; i0 < j1o && st == LA_OK; i0 += WI) {
      const int ib = std::min(WI, j1o - i0);
      const int i1 = i0 + ib;
      // One thread-block cluster holds the panel when it fits; else the
      // cooperative multi-CTA kernel.
      st = ctx->cluster_panels ? launch_panel_cluster_f32(ctx, A, ld, m, i0, ib, h->d_ipiv)
                               : LA_UNSUPPORTED;
      if (st == LA_UNSUPPORTED) st = launch_panel_f32(ctx, s, A, ld, m, i0, ib, h->d_ipiv, &bar_base);
      if (st == LA_OK) st = launch_laswp_f32(ctx, A, ld, climit, i0, ib);
      if (st == LA_OK && i1 < j1o) {
        // Two launches: fusing them into one (every CTA solving the small
        // triangle, then updating its rows from shared memory) measured 12.6 ms
        // slower at n = 16384, its update far below the GEMM tile's rate.
        st = launch_trsm_rowpanel_f32(ctx, A, ld, i0, ib, i1, j1o);
        if (st == LA_OK && i1 < m)
          st = launch_gemm_f32(ctx, GM_FMA_SUB, m - i1, j1o - i1, ib, A + (size_t)i1 * ld + i0,
                               ld, A + (size_t)i0 * ld + i1, ld, A + (size_t)i1 * ld + i1, ld);
      }
    }
    ctx->pdl_now = false;
    ctx->stream = saved;
    return st;
  };
  // U12 = L11^-1 A12 for rows [j0, j1o) on columns [c0, c1): one blocked
  // launch (the outer panel is at most 256 rows).
  auto outer_trsm = [&](int j0, int j1o, int c0, int c1) -> la_status {
    if (j1o - j0 <= 256) return launch_trsm_block_f32(ctx, A, ld, j0, j1o - j0, c0, c1);
    for (int i0 = j0; i0 < j1o; i0 += WI) {
      const int ib = std::min(WI, j1o - i0);
      const int i1 = i0 + ib;
      LA_TRY(launch_trsm_rowpanel_f32(ctx, A, ld, i0, ib, c0, c1));
      if (i1 < j1o)
        LA_TRY(launch_gemm_f32(ctx, GM_FMA_SUB, j1o - i1, c1 - c0, ib, A + (size_t)i1 * ld + i0, ld,
                               A + (size_t)i0 * ld + c0, ld, A + (size_t)i1 * ld + c0, ld));
    }
    return LA_OK;
  };
  // A22 -= L21 U12 for rows >= j1o on columns [c0, c1). L21 is copied once per
  // outer panel (pack_l) before the next panel's row swaps can permute it:
  // 16-bit K-major for the tensor cores, FP32 for the SIMT update; U12 is
  // packed per call (with its own FP16 scale).
  auto update = [&](int j0, int j1o, int c0, int c1, bool pack_l) -> la_status {
    if (c1 <= c0 || j1o >= m) return LA_OK;
    const int jbo = j1o - j0, M = m - j1o, N = c1 - c0;
    float* C = A + (size_t)j1o * ld + c0;
    if (prec == LA_PREC_FP32) {
      if (pack_l)
        LA_CUDA(ctx, cudaMemcpy2DAsync(lh.p, ldk * sizeof(float), A + (size_t)j1o * ld + j0,
                                       ld * sizeof(float), (size_t)jbo * sizeof(float), (size_t)M,
                                       cudaMemcpyDeviceToDevice, ms));
      return launch_gemm_f32(ctx, GM_FMA_SUB, M, N, jbo, lh.as<float>(), ldk,
                             A + (size_t)j0 * ld + c0, ld, C, ld);
    }
    const float* L21 = A + (size_t)j1o * ld + j0;
    const float* U12 = A + (size_t)j0 * ld + c0;
    if (prec == LA_PREC_FP8 || prec == LA_PREC_FP16X3) {
      LA_CUDA(ctx, cudaMemsetAsync(d_stat, 0, 2 * sizeof(float), ms));
      LA_CUDA(ctx, la_launch(ctx, absmax_kernel, dim3(grid_for(ctx, (size_t)jbo * N)), dim3(256), 0,
                             ms, U12, ld, jbo, N, d_stat));
      ctx->launches++;
      const dim3 pgs((N + 31) / 32, (WO + 31) / 32);
      const size_t lg = grid_for(ctx, (size_t)M * WO);
      void* ub;
      if (prec == LA_PREC_FP8) {
        uint8_t* u8 = uh.as<uint8_t>() + (size_t)(c0 - j1o) * ldks;
        ub = u8;
        if (pack_l)
          LA_CUDA(ctx, la_launch(ctx, pack_l_split_kernel<SplitE4M3>, dim3(lg), dim3(256), 0, ms,
                                 L21, ld, lh.as<uint8_t>(), ldks, M, jbo));
        LA_CUDA(ctx, la_launch(ctx, pack_ut_split_kernel<SplitE4M3>, pgs, dim3(32, 8), 0, ms, U12,
                               ld, u8, ldks, jbo, N, d_stat));
      } else {
        uint16_t* u16 = uh.as<uint16_t>() + (size_t)(c0 - j1o) * ldks;
        ub = u16;
        if (pack_l)
          LA_CUDA(ctx, la_launch(ctx, pack_l_split_kernel<SplitF16>, dim3(lg), dim3(256), 0, ms,
                                 L21, ld, lh.as<uint16_t>(), ldks, M, jbo));
        LA_CUDA(ctx, la_launch(ctx, pack_ut_split_kernel<SplitF16>, pgs, dim3(32, 8), 0, ms, U12,
                               ld, u16, ldks, jbo, N, d_stat));
      }
      ctx->launches += pack_l ? 2 : 1;
      LA_TRY(la_check_launch(ctx, "pack_split_kernel"));
      return launch_tc_update(ctx, ms, prec == LA_PREC_FP8 ? LA_LOWP_E4M3X3 : LA_LOWP_F16X3, M, N,
                              jbo, lh.p, ldks, ub, ldks, C, ld, d_stat + 1);
    }
    const int fmt = prec == LA_PREC_BF16 ? LA_LOWP_BF16 : LA_LOWP_FP16;
    uint16_t* ub = uh.as<uint16_t>() + (size_t)(c0 - j1o) * ldk;
    if (fmt == LA_LOWP_FP16) {
      LA_CUDA(ctx, cudaMemsetAsync(d_stat, 0, 2 * sizeof(float), ms));
      LA_CUDA(ctx, la_launch(ctx, absmax_kernel, dim3(grid_for(ctx, (size_t)jbo * N)), dim3(256), 0,
                             ms, U12, ld, jbo, N, d_stat));
      ctx->launches++;
    } else {
      LA_CUDA(ctx, la_launch(ctx, set_alpha_one, dim3(1), dim3(1), 0, ms, d_stat));
      ctx->launches++;
    }
    if (pack_l) {
      const dim3 lg(grid_for(ctx, (size_t)M * ldk));
      if (fmt == LA_LOWP_BF16)
        LA_CUDA(ctx, la_launch(ctx, pack_l_kernel<LA_LOWP_BF16>, lg, dim3(256), 0, ms, L21, ld,
                               lh.as<uint16_t>(), ldk, M, jbo));
      else
        LA_CUDA(ctx, la_launch(ctx, pack_l_kernel<LA_LOWP_FP16>, lg, dim3(256), 0, ms, L21, ld,
                               lh.as<uint16_t>(), ldk, M, jbo));
      ctx->launches++;
    }
    dim3 pg((N + 31) / 32, ((int)ldk + 31) / 32);
    if (fmt == LA_LOWP_BF16)
      LA_CUDA(ctx, la_launch(ctx, pack_ut_kernel<LA_LOWP_BF16>, pg, dim3(32, 8), 0, ms, U12, ld, ub,
                             ldk, jbo, N, d_stat));
    else
      LA_CUDA(ctx, la_launch(ctx, pack_ut_kernel<LA_LOWP_FP16>, pg, dim3(32, 8), 0, ms, U12, ld, ub,
                             ldk, jbo, N, d_stat));
    ctx->launches++;
    return launch_tc_update(ctx, ms, fmt, M, N, jbo, lh.p, ldk, ub, ldk, C, ld, d_stat + 1);
  };

  // No launch after this function keeps the dependent-launch attribute, also
  // on an early return.
  struct PdlReset {
    la_ctx c;
    ~PdlReset() { c->pdl_now = false; }
  } pdl_reset{ctx};
  // The first outer panel on the main stream.
  LA_TRY(inner(0, std::min(WO, kmin), std::min(WO, kmin), ms));
  for (int j0 = 0; j0 < kmin; j0 += WO) {
    const int j1o = std::min(j0 + WO, kmin);
    if (j1o >= n) break;
    const int j2o = std::min(j1o + WO, kmin);  // the next outer panel [j1o, j2o)
    // This panel's swaps on the columns its inner panels left out, then the
    // next panel's columns: the serial part between the two chains, as
    // dependent launches (the rest of the update, after the fork, is not).
    ctx->pdl_now = ctx->pdl != 0;
    LA_TRY(launch_laswp_seq_f32(ctx, A, ld, h->d_ipiv, j0, j1o, j1o, n));
    LA_TRY(outer_trsm(j0, j1o, j1o, j2o));
    LA_TRY(update(j0, j1o, j1o, j2o, true));
    ctx->pdl_now = false;
    bool forked = false;
    if (j1o < kmin) {
      if (look) {
        LA_CUDA(ctx, cudaEventRecord(ctx->ev_fork, ms));
        LA_CUDA(ctx, cudaStreamWaitEvent(ss, ctx->ev_fork, 0));
      }
      LA_TRY(inner(j1o, j2o, j2o, ss));
      forked = look;
    }
    if (j2o < n) {
      // One launch each for the rest (splitting it into column chunks, to let
      // the side stream's panels in between, measured 9-14 % slower).
      LA_TRY(outer_trsm(j0, j1o, j2o, n));
      LA_TRY(update(j0, j1o, j2o, n, false));
    }
    if (forked) {
      LA_CUDA(ctx, cudaEventRecord(ctx->ev_join, ss));
      LA_CUDA(ctx, cudaStreamWaitEvent(ms, ctx->ev_join, 0));
    }
  }
  return LA_OK;
}

// Iterative refinement with the mixed factors of h (la_lu_solve_refined_device;
// allow_gmres = false stops when plain refinement stalls).
la_status refine_impl(la_lu h, const double* d_b, size_t ldb, size_t nrhs, double* d_x,
                      size_t ldx, int max_iters, double tol, bool allow_gmres,
                      la_refine_stats* stats);

}  // namespace

extern "C" {

la_status la_lu_mixed_new_device(la_ctx ctx, const double* d_a, size_t lda, size_t n, int prec,
                                 la_lu* out) {
  if (!ctx || !d_a || !out || lda < n) return LA_INVALID;
  if (n == 0) return LA_BADSHAPE;
  if (n > (size_t)INT32_MAX / 4) return LA_UNSUPPORTED;
  if (prec != LA_PREC_BF16 && prec != LA_PREC_FP16 && prec != LA_PREC_FP32 &&
      prec != LA_PREC_FP8 && prec != LA_PREC_FP16X3)
    return LA_INVALID;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  *out = nullptr;
  la_lu h = new (std::nothrow) la_lu_handle();
  if (!h) return LA_NOMEM;
  h->ctx = ctx;
  h->m = h->n = n;
  h->ld = (n + 3) & ~size_t(3);
  h->ld32 = pad8(n);
  h->lowp = prec;
  h->arith = LA_ARITH_FAST;
  void* p = nullptr;
  la_status s = la_device_alloc(ctx, &p, n * h->ld * sizeof(double));
  if (s == LA_OK) { h->d_lu = static_cast<double*>(p); s = la_device_alloc(ctx, &p, n * h->ld32 * 4); }
  if (s == LA_OK) { h->d_lu32 = static_cast<float*>(p); s = la_device_alloc(ctx, &p, n * sizeof(int)); }
  if (s == LA_OK) { h->d_ipiv = static_cast<int*>(p); s = la_device_alloc(ctx, &p, n * 8); }
  if (s == LA_OK) h->d_piv = static_cast<uint64_t*>(p);
  if (s != LA_OK) { la_lu_free(h); return s; }
  cudaError_t e = cudaMemcpy2DAsync(h->d_lu, h->ld * 8, d_a, lda * 8, n * 8, n,
                                    cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) { s = la_cuda_fail(ctx, e, "copy A"); la_lu_free(h); return s; }
  f64_to_f32_kernel<<<grid_for(ctx, n * n), 256, 0, ctx->stream>>>(h->d_lu, h->ld, h->d_lu32,
                                                                    h->ld32, (int)n, (int)n);
  ctx->launches++;
  s = la_check_launch(ctx, "f64_to_f32_kernel");
  if (s == LA_OK) s = mixed_factor(ctx, h, prec);
  if (s == LA_OK) s = launch_lu_finish(ctx, h, reinterpret_cast<int*>(ctx->d_small));
  int* flags = static_cast<int*>(ctx->h_pinned);
  if (s == LA_OK) {
    e = cudaMemcpyAsync(flags, ctx->d_small, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) s = la_cuda_fail(ctx, e, "flags");
  }
  if (s == LA_OK) s = la_sync_and_check(ctx, "mixed factorization");
  if (s != LA_OK) { la_lu_free(h); return s; }
  h->pospivsign = flags[0];
  h->zero_diag = flags[1];
  *out = h;
  return LA_OK;
}

la_status la_lu_solve_refined_device(la_lu h, const double* d_b, size_t ldb, size_t nrhs,
                                     double* d_x, size_t ldx, int max_iters, double tol,
                                     la_refine_stats* stats) {
  return refine_impl(h, d_b, ldb, nrhs, d_x, ldx, max_iters, tol, true, stats);
}

la_status la_lu_solve_auto_device(la_ctx ctx, const double* d_a, size_t lda, size_t n,
                                  const double* d_b, size_t ldb, size_t nrhs, double* d_x,
                                  size_t ldx, double tol, la_refine_stats* stats) {
  if (!ctx || !d_a || !d_b || !d_x || lda < n || ldb < nrhs || ldx < nrhs) return LA_INVALID;
  if (n == 0) return LA_BADSHAPE;
  if (nrhs == 0 || nrhs > 16) return LA_UNSUPPORTED;
  la_refine_stats st = {};
  int its = 0;
  // 1. Split-FP16 trailing updates (three tensor-core products per term):
  //    factors close to FP32 quality at the cost of the FP16 update, which is
  //    bound by the read-modify-write of the trailing matrix, not by the
  //    tensor pipe. Plain refinement, then GMRES-IR if it stalls. Measured
  //    at n = 16384 it beats single FP16 factors (fewer refinement steps) and
  //    the FP32 SIMT factorization at every condition number tried, so no
  //    cheaper stage comes first and no condition estimate is needed to skip
  //    one.
  {
    la_lu h = nullptr;
    la_status s = la_lu_mixed_new_device(ctx, d_a, lda, n, LA_PREC_FP16X3, &h);
    if (s != LA_OK) return s;
    s = refine_impl(h, d_b, ldb, nrhs, d_x, ldx, 40, tol, true, &st);
    la_lu_free(h);
    its += s == LA_SINGULAR ? 0 : st.iterations;
    if (s == LA_OK) {
      st.iterations = its;
      st.fell_back = 0;
      if (stats) *stats = st;
      return LA_OK;
    }
    if (s != LA_NOT_CONVERGED && s != LA_SINGULAR) return s;
  }
  // 2. The plain FP64 LU (the reference's algorithm) answers, and decides: a
  //    zero pivot there is the reference's None.
  la_lu lu = nullptr;
  la_status s = la_lu_new_device(ctx, d_a, lda, n, n, &lu);
  if (s != LA_OK) return s;
  s = la_lu_solve_device(lu, d_b, ldb, n, nrhs, d_x, ldx);
  la_lu_free(lu);
  if (s != LA_OK) return s;
  double eta = 0.0;
  LA_TRY(la_backward_error_device(ctx, d_a, lda, d_x, ldx, d_b, ldb, n, nrhs, &eta));
  st.iterations = its;
  st.converged = eta <= tol ? 1 : 0;
  st.eta = eta;
  st.fell_back = 1;
  st.precision = 0;
  st.gmres_steps = 0;
  if (stats) *stats = st;
  return LA_OK;
}

}  // extern "C"

namespace {

la_status refine_impl(la_lu h, const double* d_b, size_t ldb, size_t nrhs, double* d_x,
                      size_t ldx, int max_iters, double tol, bool allow_gmres,
                      la_refine_stats* stats) {
  if (!h || !d_b || !d_x || ldb < nrhs || ldx < nrhs || !h->d_lu32) return LA_INVALID;
  if (nrhs == 0 || nrhs > 16) return LA_UNSUPPORTED;
  la_ctx ctx = h->ctx;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  if (h->zero_diag) return LA_SINGULAR;
  const int n = (int)h->n, R = (int)nrhs;
  cudaStream_t st = ctx->stream;
  const size_t ldw = 4 * ((nrhs + 3) / 4);
  Buf rbuf(ctx), wbuf(ctx), norms(ctx), sync(ctx);
  LA_TRY(rbuf.alloc((size_t)n * nrhs * 8));
  LA_TRY(wbuf.alloc((size_t)n * ldw * 4));
  const int nb64 = (n + 63) / 64;
  LA_TRY(sync.alloc((size_t)(2 * nb64 + 2) * sizeof(int)));
  LA_TRY(ensure_dinv(ctx, h));
  // norms: [0] ||A||, [8..8+R) rmax, [32..32+R) xmax, [56..56+R) bmax
  LA_TRY(norms.alloc(128 * 8));
  double* d_norm = norms.as<double>();
  double* d_r = rbuf.as<double>();
  float* d_w = wbuf.as<float>();
  LA_CUDA(ctx, cudaMemsetAsync(d_norm, 0, 128 * 8, st));
  rownorm_kernel<<<grid_for(ctx, (size_t)n * 32), 256, 0, st>>>(h->d_lu, h->ld, n, d_norm);
  colmax_kernel<<<grid_for(ctx, (size_t)n * nrhs), 256, 0, st>>>(d_b, ldb, n, R, d_norm + 56);
  ctx->launches += 2;
  // x = 0, r = b
  LA_CUDA(ctx, cudaMemset2DAsync(d_x, ldx * 8, 0, nrhs * 8, n, st));
  LA_CUDA(ctx, cudaMemcpy2DAsync(d_r, nrhs * 8, d_b, ldb * 8, nrhs * 8, n,
                                 cudaMemcpyDeviceToDevice, st));
  LA_CUDA(ctx, cudaMemcpyAsync(d_norm + 8, d_norm + 56, R * 8, cudaMemcpyDeviceToDevice, st));
  double* host = static_cast<double*>(ctx->h_pinned);
  double eta_col[16];
  double eta = INFINITY;
  // eta from the current r (norms in d_norm) and x.
  auto measure = [&]() -> la_status {
    LA_CUDA(ctx, cudaMemsetAsync(d_norm + 32, 0, 16 * 8, st));
    colmax_kernel<<<grid_for(ctx, (size_t)n * nrhs), 256, 0, st>>>(d_x, ldx, n, R, d_norm + 32);
    ctx->launches++;
    LA_CUDA(ctx, cudaMemcpyAsync(host, d_norm, 72 * 8, cudaMemcpyDeviceToHost, st));
    LA_TRY(la_sync_and_check(ctx, "refinement norms"));
    eta = 0.0;
    for (int j = 0; j < R; j++) {
      const double den = host[0] * host[32 + j] + host[56 + j];
      const double v = den > 0 ? host[8 + j] / den : (host[8 + j] > 0 ? INFINITY : 0.0);
      eta_col[j] = v;
      if (!(v <= eta)) eta = v;
    }
    return LA_OK;
  };
  // r = b - A x and its column maxima.
  auto residual = [&]() -> la_status {
    LA_CUDA(ctx, cudaMemsetAsync(d_norm + 8, 0, 16 * 8, st));
    launch_residual(n, R, st, h->d_lu, h->ld, d_x, ldx, d_b, ldb, d_r, nrhs, d_norm + 8);
    ctx->launches++;
    return la_check_launch(ctx, "residual");
  };
  LA_TRY(measure());
  double prev = INFINITY;
  int it = 0, gsteps = 0;
  bool converged = eta <= tol;
  // A stall injected for tests (LA_OPT_INJECT_IR_STALL): no correction runs.
  bool stall = false;
  if (ctx->inject_ir_stall > 0) {
    ctx->inject_ir_stall--;
    stall = true;
  }
  // Plain refinement: d = LU32 \ (r(piv) / rmax), x += d * rmax.
  while (!stall && !converged && it < max_iters && eta < 0.9 * prev) {
    prev = eta;
    it++;
    scale_permute_kernel<<<grid_for(ctx, (size_t)n * nrhs), 256, 0, st>>>(
        h->d_piv, d_r, nrhs, d_norm + 8, d_w, ldw, n, R);
    ctx->launches++;
    LA_TRY(launch_trsv_wave_f32f(ctx, h->d_lu32, h->ld32, h->d_dinvf, d_w, ldw, n, R,
                                 sync.as<int>()));
    update_x_kernel<<<grid_for(ctx, (size_t)n * nrhs), 256, 0, st>>>(d_x, ldx, d_w, ldw,
                                                                      d_norm + 8, n, R);
    ctx->launches++;
    LA_TRY(residual());
    LA_TRY(measure());
    converged = eta <= tol;
  }
  // GMRES-IR once plain refinement stalls.
  int outer = 0;
  prev = INFINITY;
  while (!stall && allow_gmres && !converged && it + outer < max_iters && eta < 0.5 * prev) {
    prev = eta;
    outer++;
    for (int j = 0; j < R; j++) {
      if (eta_col[j] <= tol) continue;
      int steps = 0;
      LA_TRY(gmres_correction(ctx, h, d_r, nrhs, j, d_x, ldx, 60, 1e-10, &steps));
      gsteps += steps;
    }
    LA_TRY(residual());
    LA_TRY(measure());
    converged = eta <= tol;
  }
  if (stats) {
    stats->iterations = it + outer;
    stats->eta = eta;
    stats->converged = converged ? 1 : 0;
    stats->gmres_steps = gsteps;
    stats->precision = h->lowp;
    stats->fell_back = 0;
  }
  return converged ? LA_OK : LA_NOT_CONVERGED;
}

}  // namespace
