// Row swaps, triangular updates and the small kernels around the blocked LU.
#include "la_internal.cuh"

namespace {

// ---- row swaps outside the panel (lu.rs:140-145 for the other columns) ----
// Applies the composed moves of one panel (dest <- src) to columns
// [c_begin, c_end) of one matrix. All sources are read into shared memory
// before any destination is written, so the moves act as one permutation.
constexpr int SW_COLS = 32;

// The context's error word (nonzero after a device wait gave up). The kernels
// that apply a panel's row interchanges return at entry when it is set: a
// panel that gave up left no valid interchanges behind.
__device__ __forceinline__ bool aborted(const int* err) {
  return err != nullptr && *reinterpret_cast<const volatile int*>(err) != 0;
}

template <typename T>
__global__ void __launch_bounds__(256)
laswp_kernel(T* M0, T* M1, T* M2, size_t ld, int b0, int e0, int b1, int e1,
             int b2, int e2, const int* __restrict__ swaps, const int* err) {
  la_pdl_wait();
  la_pdl_trigger();
  __shared__ T tmp[2 * MAX_PANEL_W][SW_COLS];
  __shared__ int s_abort;
  if (threadIdx.x == 0) s_abort = aborted(err);
  __syncthreads();
  if (s_abort) return;
  const int cnt = swaps[0];
  if (cnt == 0) return;
  const int* dst = swaps + 1;
  const int* src = swaps + 1 + 2 * MAX_PANEL_W;
  // blockIdx.y selects the segment.
  T* M;
  int cb, ce;
  if (blockIdx.y == 0) { M = M0; cb = b0; ce = e0; }
  else if (blockIdx.y == 1) { M = M1; cb = b1; ce = e1; }
  else { M = M2; cb = b2; ce = e2; }
  if (M == nullptr) return;
  const int c = cb + blockIdx.x * SW_COLS + (threadIdx.x % SW_COLS);
  if (cb + (int)blockIdx.x * SW_COLS >= ce) return;
  const int ty = threadIdx.x / SW_COLS;  // 0..7
  const bool ok = c < ce;
  for (int q = ty; q < cnt; q += 8)
    if (ok) tmp[q][threadIdx.x % SW_COLS] = M[(size_t)src[q] * ld + c];
  __syncthreads();
  for (int q = ty; q < cnt; q += 8)
    if (ok) M[(size_t)dst[q] * ld + c] = tmp[q][threadIdx.x % SW_COLS];
}

// Row interchanges of pivot positions [k0, k1) (ipiv[k] = the row swapped with
// row k, in order) on columns [c0, c1): one thread per column applies the swaps
// in sequence (the panel's own composed moves are for the columns next to the
// panel; this form serves columns whose swaps were deferred).
template <typename T>
__global__ void laswp_seq_kernel(T* A, size_t ld, const int* __restrict__ ipiv, int k0, int k1,
                                 int c0, int c1, const int* err) {
  la_pdl_wait();
  la_pdl_trigger();
  const int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= c1 || aborted(err)) return;  // no barrier in this kernel
  for (int k = k0; k < k1; k++) {
    const int p = ipiv[k];
    if (p != k) {
      T* a = A + (size_t)k * ld + c;
      T* b = A + (size_t)p * ld + c;
      const T t = *a;
      *a = *b;
      *b = t;
    }
  }
}

// ---- row-panel triangular update: U12 = L11^{-1} A12 ----------------------
// Rows [j0, j0+jb), columns [c_begin, c_end), one 32-column strip per CTA.
// Column sweep over k (one barrier per k): row k is finished, then every row
// i > k of the block takes its k-th term, i.e. each element receives its terms
// in ascending k, like lu.rs:124-128 (EXACT: s += l*u, u = a - s) or with FMA.
constexpr int TR_COLS = 32;
constexpr int LP = MAX_PANEL_W + 1;  // padded row of the triangular block in shared memory
template <typename T>
constexpr size_t trsm_smem(bool exact) {
  return (size_t)(MAX_PANEL_W * LP + MAX_PANEL_W * TR_COLS * (exact ? 2 : 1)) * sizeof(T);
}

template <typename T, bool EXACT>
__global__ void __launch_bounds__(256)
trsm_rowpanel_kernel(T* A, const T* S, size_t ld, int j0, int jb, int c_begin, int c_end) {
  extern __shared__ __align__(16) double dsm_raw[];
  T* dsm = reinterpret_cast<T*>(dsm_raw);
  T(*L)[LP] = reinterpret_cast<T(*)[LP]>(dsm);
  T(*xa)[TR_COLS] = reinterpret_cast<T(*)[TR_COLS]>(dsm + MAX_PANEL_W * LP);
  T(*xs)[TR_COLS] =
      reinterpret_cast<T(*)[TR_COLS]>(dsm + MAX_PANEL_W * LP + MAX_PANEL_W * TR_COLS);
  const int tx = threadIdx.x % TR_COLS, ty = threadIdx.x / TR_COLS;  // ty 0..7
  const int c = c_begin + blockIdx.x * TR_COLS + tx;
  const bool ok = c < c_end;
  for (int idx = threadIdx.x; idx < jb * jb; idx += 256) {
    int i = idx / jb, k = idx % jb;
    L[i][k] = A[(size_t)(j0 + i) * ld + j0 + k];
  }
  for (int i = ty; i < jb; i += 8) {
    size_t off = (size_t)(j0 + i) * ld + c;
    xa[i][tx] = ok ? A[off] : T(0);
    if (EXACT) xs[i][tx] = ok ? S[off] : T(0);
  }
  __syncthreads();
  for (int k = 0; k < jb; k++) {
    if (EXACT && ty == (k & 7)) {
      // Row k is complete (this thread applied all its earlier terms): u = a - s.
      xa[k][tx] = __dsub_rn(xa[k][tx], xs[k][tx]);
    }
    __syncthreads();
    const T uk = xa[k][tx];
    for (int i = ty; i < jb; i += 8) {
      if (i <= k) continue;
      if (EXACT)
        xs[i][tx] = __dadd_rn(xs[i][tx], __dmul_rn(L[i][k], uk));
      else
        xa[i][tx] = fma(-L[i][k], uk, xa[i][tx]);
    }
  }
  __syncthreads();
  if (ok)
    for (int i = ty; i < jb; i += 8) A[(size_t)(j0 + i) * ld + c] = xa[i][tx];
}

// FP32 form for the mixed LU's 32-row blocks (jb <= 32, FMA): one thread per
// column holds the column's jb values in registers and applies the terms in
// ascending k (the same FMAs in the same order as the kernel above, so the
// same bits), with the unit-lower block broadcast from shared memory. No
// barrier inside the sweep: at FP32 rates the barriers, not the FMAs, were the
// cost of the 32-step sweep.
constexpr int TRR_W = 32;
constexpr int TRR_T = 128;
__global__ void __launch_bounds__(TRR_T)
trsm_rowpanel_reg_kernel(float* A, size_t ld, int j0, int jb, int c_begin, int c_end) {
  la_pdl_wait();
  la_pdl_trigger();
  __shared__ float L[TRR_W][TRR_W + 1];
  for (int idx = threadIdx.x; idx < jb * jb; idx += TRR_T) {
    const int i = idx / jb, k = idx % jb;
    L[i][k] = A[(size_t)(j0 + i) * ld + j0 + k];
  }
  __syncthreads();
  const int c = c_begin + blockIdx.x * TRR_T + threadIdx.x;
  if (c >= c_end) return;
  float x[TRR_W];
#pragma unroll
  for (int i = 0; i < TRR_W; i++) x[i] = i < jb ? A[(size_t)(j0 + i) * ld + c] : 0.f;
#pragma unroll
  for (int k = 0; k < TRR_W; k++) {
    if (k >= jb) break;
    const float xk = x[k];
#pragma unroll
    for (int i = k + 1; i < TRR_W; i++)
      if (i < jb) x[i] = fmaf(-L[i][k], xk, x[i]);
  }
#pragma unroll
  for (int i = 0; i < TRR_W; i++)
    if (i < jb) A[(size_t)(j0 + i) * ld + c] = x[i];
}

// ---- the mixed LU's outer-panel triangular update: X = L11^-1 X ----------------------
// Rows [j0, j0 + jbo) (jbo <= 256) of columns [c_begin, c_end), L11 the unit
// lower jbo x jbo block of A at (j0, j0). One CTA per 32 columns keeps its
// jbo x 32 block of X in shared memory. Per 32-row block of L11: the block's
// rows and everything below it in its 32 columns are staged in shared memory;
// warp 0 solves the diagonal block (lane = column, the 32 values in registers,
// no barrier inside); then the 256 threads subtract the block's contribution
// from the rows below (8 threads per row, 4 columns each, 32-deep dot products
// from shared memory). One launch instead of a row-panel solve and a GEMM per
// 32 rows.
constexpr int TB_R = 256, TB_C = 32;
constexpr size_t TB_SMEM = (size_t)2 * TB_R * (TB_C + 1) * sizeof(float);
__global__ void __launch_bounds__(256)
trsm_block_kernel(float* A, size_t ld, int j0, int jbo, int c_begin, int c_end) {
  la_pdl_wait();
  la_pdl_trigger();
  extern __shared__ __align__(16) float tb_sm[];
  float(*X)[TB_C + 1] = reinterpret_cast<float(*)[TB_C + 1]>(tb_sm);
  float(*Lb)[TB_C + 1] = reinterpret_cast<float(*)[TB_C + 1]>(tb_sm + TB_R * (TB_C + 1));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cb = c_begin + blockIdx.x * TB_C;
  for (int idx = tid; idx < jbo * TB_C; idx += 256) {
    const int r = idx / TB_C, c = idx % TB_C;
    X[r][c] = cb + c < c_end ? A[(size_t)(j0 + r) * ld + cb + c] : 0.f;
  }
  for (int kb = 0; kb < jbo; kb += TB_C) {
    const int bw = min(TB_C, jbo - kb);
    // L11 rows [kb, jbo) of columns [kb, kb + bw)
    for (int idx = tid; idx < (jbo - kb) * TB_C; idx += 256) {
      const int r = idx / TB_C, k = idx % TB_C;
      Lb[r][k] = k < bw ? A[(size_t)(j0 + kb + r) * ld + j0 + kb + k] : 0.f;
    }
    __syncthreads();
    if (warp == 0) {
      float x[TB_C];
#pragma unroll
      for (int i = 0; i < TB_C; i++) x[i] = i < bw ? X[kb + i][lane] : 0.f;
#pragma unroll
      for (int k = 0; k < TB_C; k++) {
        if (k >= bw) break;
        const float xk = x[k];
#pragma unroll
        for (int i = k + 1; i < TB_C; i++) x[i] = fmaf(-Lb[i][k], xk, x[i]);
      }
#pragma unroll
      for (int i = 0; i < TB_C; i++)
        if (i < bw) X[kb + i][lane] = x[i];
    }
    __syncthreads();
    const int rows = jbo - kb - bw;
    for (int e = tid; e < rows * 8; e += 256) {
      const int r = e >> 3, c4 = (e & 7) * 4, i = kb + bw + r;
      float a0 = X[i][c4], a1 = X[i][c4 + 1], a2 = X[i][c4 + 2], a3 = X[i][c4 + 3];
      for (int k = 0; k < bw; k++) {
        const float l = Lb[bw + r][k];
        a0 = fmaf(-l, X[kb + k][c4], a0);
        a1 = fmaf(-l, X[kb + k][c4 + 1], a1);
        a2 = fmaf(-l, X[kb + k][c4 + 2], a2);
        a3 = fmaf(-l, X[kb + k][c4 + 3], a3);
      }
      X[i][c4] = a0;
      X[i][c4 + 1] = a1;
      X[i][c4 + 2] = a2;
      X[i][c4 + 3] = a3;
    }
    __syncthreads();
  }
  for (int idx = tid; idx < jbo * TB_C; idx += 256) {
    const int r = idx / TB_C, c = idx % TB_C;
    if (cb + c < c_end) A[(size_t)(j0 + r) * ld + cb + c] = X[r][c];
  }
}

// ---- after the factorization: permutation vector, sign, zero diagonal ------
// The swap list (LAPACK ipiv form) is replayed in order on a permutation
// vector (lu.rs:147-149), the sign flips once per real swap (lu.rs:151), and
// U's diagonal is scanned for an exact zero (lu.rs:177).
template <typename T>
__global__ void lu_finish_kernel(const int* __restrict__ ipiv, uint64_t* piv, int m, int kmin,
                                 const T* LU, size_t ld, int* flags, int smem_rows,
                                 const int* err) {
  extern __shared__ int sperm[];  // permutation in shared memory when m fits
  __shared__ int zero, s_abort;
  if (threadIdx.x == 0) s_abort = aborted(err);
  __syncthreads();
  if (s_abort) return;  // the host reports the error; flags and piv are not used
  if (threadIdx.x == 0) zero = 0;
  const bool in_smem = m <= smem_rows;
  if (in_smem) {
    for (int i = threadIdx.x; i < m; i += blockDim.x) sperm[i] = i;
  } else {
    for (int i = threadIdx.x; i < m; i += blockDim.x) piv[i] = (uint64_t)i;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < kmin; j += blockDim.x)
    if (LU[(size_t)j * ld + j] == T(0)) atomicOr(&zero, 1);
  if (threadIdx.x == 0) {
    int pos = 1;
    for (int j = 0; j < kmin; j++) {
      int p = ipiv[j];
      if (p != j) {
        if (in_smem) {
          int t = sperm[p];
          sperm[p] = sperm[j];
          sperm[j] = t;
        } else {
          uint64_t t = piv[p];
          piv[p] = piv[j];
          piv[j] = t;
        }
        pos = !pos;
      }
    }
    flags[0] = pos;
  }
  __syncthreads();
  if (in_smem)
    for (int i = threadIdx.x; i < m; i += blockDim.x) piv[i] = (uint64_t)sperm[i];
  if (threadIdx.x == 0) flags[1] = zero;
}

// X = B(piv, :) (lu.rs:245-254).
__global__ void permute_rows_kernel(const uint64_t* __restrict__ piv, const double* __restrict__ B,
                                    size_t ldb, double* __restrict__ X, size_t ldx, int m,
                                    int nrhs) {
  size_t total = (size_t)m * nrhs;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(idx / nrhs), j = (int)(idx % nrhs);
    X[(size_t)i * ldx + j] = B[(size_t)piv[i] * ldb + j];
  }
}

// X = I(piv, :) for inverse (mod.rs:1036 solves against Matrix::id).
__global__ void identity_permuted_kernel(const uint64_t* __restrict__ piv, double* X, size_t ldx,
                                         int m) {
  size_t total = (size_t)m * m;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(idx / m), j = (int)(idx % m);
    X[(size_t)i * ldx + j] = (piv[i] == (uint64_t)j) ? 1.0 : 0.0;
  }
}

// det (lu.rs:224-232): one thread multiplies U's diagonal in ascending order,
// the reference's exact sequence of roundings.
__global__ void det_kernel(const double* LU, size_t ld, int n, int pospivsign, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double d = pospivsign ? 1.0 : -1.0;
    for (int j = 0; j < n; j++) d = d * LU[(size_t)j * ld + j];
    out[0] = d;
  }
}

// get_l (which 0, lu.rs:184-202), get_u (1, :204-215), get_p (2, :217-220),
// packed copy (3).
__global__ void unpack_kernel(int which, const double* LU, size_t ld, int m, int n,
                              const uint64_t* piv, double* out) {
  const int kmin = m < n ? m : n;
  int rows, cols;
  if (which == 0) { rows = m; cols = kmin; }
  else if (which == 1) { rows = kmin; cols = n; }
  else if (which == 2) { rows = m; cols = m; }
  else { rows = m; cols = n; }
  size_t total = (size_t)rows * cols;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(idx / cols), j = (int)(idx % cols);
    double v;
    if (which == 0) v = i > j ? LU[(size_t)i * ld + j] : (i == j ? 1.0 : 0.0);
    else if (which == 1) v = i <= j ? LU[(size_t)i * ld + j] : 0.0;
    else if (which == 2) v = (piv[i] == (uint64_t)j) ? 1.0 : 0.0;
    else v = LU[(size_t)i * ld + j];
    out[idx] = v;
  }
}

__global__ void copy2d_kernel(const double* __restrict__ src, size_t lds, double* __restrict__ dst,
                              size_t ldd, int rows, int cols) {
  size_t total = (size_t)rows * cols;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
       idx += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(idx / cols), j = (int)(idx % cols);
    dst[(size_t)i * ldd + j] = src[(size_t)i * lds + j];
  }
}

// Dynamic shared memory above 48 KB needs an opt-in per kernel.
cudaError_t configure_smem_attrs() {
  static la_device_once once;
  return once.run([](int) {
    cudaError_t e = cudaFuncSetAttribute(trsm_rowpanel_kernel<double, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)trsm_smem<double>(true));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(trsm_rowpanel_kernel<double, false>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)trsm_smem<double>(false));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(trsm_rowpanel_kernel<float, false>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)trsm_smem<float>(false));
    return e;
  });
}

int grid_for(la_ctx ctx, size_t total) {
  size_t g = (total + 255) / 256;
  size_t cap = (size_t)ctx->sm_count * 8;
  return (int)std::max<size_t>(1, std::min(g, cap));
}

}  // namespace

template <typename T>
la_status launch_laswp_t(la_ctx ctx, cudaStream_t stream, bool exact, T* A, T* S, size_t ld,
                         int n, int j0, int jb) {
  const int j1 = j0 + jb;
  const int left = j0, right = n - j1;
  const int gx = std::max((left + SW_COLS - 1) / SW_COLS, (right + SW_COLS - 1) / SW_COLS);
  if (gx == 0) return LA_OK;
  dim3 grid(gx, exact ? 3 : 2);
  const cudaError_t e = la_launch(ctx, laswp_kernel<T>, grid, dim3(256), 0, stream, A, A,
                                  exact ? S : nullptr, ld, 0, j0, j1, n, j1, n,
                                  (const int*)ctx->d_swaps, (const int*)ctx->d_err);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "laswp_kernel launch");
  ctx->launches++;
  return la_check_launch(ctx, "laswp_kernel");
}

la_status launch_laswp(la_ctx ctx, bool exact, double* A, double* S, size_t ld, int n, int j0,
                       int jb) {
  return launch_laswp_t<double>(ctx, ctx->stream, exact, A, S, ld, n, j0, jb);
}
la_status launch_laswp_f32(la_ctx ctx, float* A, size_t ld, int n, int j0, int jb) {
  return launch_laswp_t<float>(ctx, ctx->stream, false, A, nullptr, ld, n, j0, jb);
}
la_status launch_trsm_block_f32(la_ctx ctx, float* A, size_t ld, int j0, int jbo, int c_begin,
                                int c_end) {
  if (c_end <= c_begin || jbo <= 0) return LA_OK;
  if (jbo > TB_R) return LA_INVALID;
  static la_device_once once;
  LA_CUDA(ctx, once.run([](int) {
            return cudaFuncSetAttribute(trsm_block_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)TB_SMEM);
          }));
  const cudaError_t e = la_launch(ctx, trsm_block_kernel, dim3((c_end - c_begin + TB_C - 1) / TB_C),
                                  dim3(256), TB_SMEM, ctx->stream, A, ld, j0, jbo, c_begin, c_end);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "trsm_block_kernel launch");
  ctx->launches++;
  return la_check_launch(ctx, "trsm_block_kernel");
}

la_status launch_laswp_seq_f32(la_ctx ctx, float* A, size_t ld, const int* ipiv, int k0, int k1,
                               int c0, int c1) {
  if (k1 <= k0 || c1 <= c0) return LA_OK;
  const cudaError_t e = la_launch(ctx, laswp_seq_kernel<float>, dim3((c1 - c0 + 255) / 256),
                                  dim3(256), 0, ctx->stream, A, ld, ipiv, k0, k1, c0, c1,
                                  (const int*)ctx->d_err);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "laswp_seq_kernel launch");
  ctx->launches++;
  return la_check_launch(ctx, "laswp_seq_kernel");
}

template <typename T>
la_status launch_trsm_t(la_ctx ctx, bool exact, T* A, T* S, size_t ld, int j0, int jb,
                        int c_begin, int c_end) {
  if (c_end <= c_begin) return LA_OK;
  LA_CUDA(ctx, configure_smem_attrs());
  dim3 grid((c_end - c_begin + TR_COLS - 1) / TR_COLS);
  if (exact)
    trsm_rowpanel_kernel<T, true><<<grid, 256, trsm_smem<T>(true), ctx->stream>>>(A, S, ld, j0, jb,
                                                                               c_begin, c_end);
  else
    trsm_rowpanel_kernel<T, false><<<grid, 256, trsm_smem<T>(false), ctx->stream>>>(
        A, S, ld, j0, jb, c_begin, c_end);
  ctx->launches++;
  return la_check_launch(ctx, "trsm_rowpanel_kernel");
}

la_status launch_trsm_rowpanel(la_ctx ctx, bool exact, double* A, double* S, size_t ld, int j0,
                               int jb, int c_begin, int c_end) {
  return launch_trsm_t<double>(ctx, exact, A, S, ld, j0, jb, c_begin, c_end);
}
la_status launch_trsm_rowpanel_f32(la_ctx ctx, float* A, size_t ld, int j0, int jb, int c_begin,
                                   int c_end) {
  if (jb > TRR_W) return launch_trsm_t<float>(ctx, false, A, nullptr, ld, j0, jb, c_begin, c_end);
  if (c_end <= c_begin) return LA_OK;
  const int grid = (c_end - c_begin + TRR_T - 1) / TRR_T;
  const cudaError_t e = la_launch(ctx, trsm_rowpanel_reg_kernel, dim3(grid), dim3(TRR_T), 0,
                                  ctx->stream, A, ld, j0, jb, c_begin, c_end);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "trsm_rowpanel_reg_kernel launch");
  ctx->launches++;
  return la_check_launch(ctx, "trsm_rowpanel_reg_kernel");
}

la_status launch_lu_finish(la_ctx ctx, la_lu h, int* d_flags) {
  const int kmin = (int)std::min(h->m, h->n);
  const int smem_rows = 50000;  // 200 KB of int32 (opt-in); larger m replays in global memory
  static la_device_once configured;
  cudaError_t ce = configured.run([&](int) {
    cudaError_t e = cudaFuncSetAttribute(lu_finish_kernel<double>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         smem_rows * (int)sizeof(int));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(lu_finish_kernel<float>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               smem_rows * (int)sizeof(int));
    return e;
  });
  if (ce != cudaSuccess) return la_cuda_fail(ctx, ce, "cudaFuncSetAttribute(lu_finish)");
  const size_t smem = (size_t)std::min((int)h->m, smem_rows) * sizeof(int);
  if (h->d_lu32)
    lu_finish_kernel<float><<<1, 1024, smem, ctx->stream>>>(h->d_ipiv, h->d_piv, (int)h->m, kmin,
                                                            h->d_lu32, h->ld32, d_flags, smem_rows,
                                                            ctx->d_err);
  else
    lu_finish_kernel<double><<<1, 1024, smem, ctx->stream>>>(h->d_ipiv, h->d_piv, (int)h->m, kmin,
                                                             h->d_lu, h->ld, d_flags, smem_rows,
                                                             ctx->d_err);
  ctx->launches++;
  return la_check_launch(ctx, "lu_finish_kernel");
}

la_status launch_permute_rows(la_ctx ctx, const uint64_t* d_piv, const double* B, size_t ldb,
                              double* X, size_t ldx, int m, int nrhs) {
  permute_rows_kernel<<<grid_for(ctx, (size_t)m * nrhs), 256, 0, ctx->stream>>>(d_piv, B, ldb, X,
                                                                               ldx, m, nrhs);
  ctx->launches++;
  return la_check_launch(ctx, "permute_rows_kernel");
}

la_status launch_identity_permuted(la_ctx ctx, const uint64_t* d_piv, double* X, size_t ldx,
                                   int m) {
  identity_permuted_kernel<<<grid_for(ctx, (size_t)m * m), 256, 0, ctx->stream>>>(d_piv, X, ldx,
                                                                                  m);
  ctx->launches++;
  return la_check_launch(ctx, "identity_permuted_kernel");
}

la_status launch_det(la_ctx ctx, const double* LU, size_t ld, int n, int pospivsign,
                     double* d_out) {
  det_kernel<<<1, 32, 0, ctx->stream>>>(LU, ld, n, pospivsign, d_out);
  ctx->launches++;
  return la_check_launch(ctx, "det_kernel");
}

la_status launch_unpack(la_ctx ctx, int which, const double* LU, size_t ld, int m, int n,
                        const uint64_t* d_piv, double* out) {
  size_t total = (size_t)std::max(m, n) * std::max(m, n);
  unpack_kernel<<<grid_for(ctx, total), 256, 0, ctx->stream>>>(which, LU, ld, m, n, d_piv, out);
  ctx->launches++;
  return la_check_launch(ctx, "unpack_kernel");
}

la_status launch_copy2d(la_ctx ctx, const double* src, size_t lds, double* dst, size_t ldd,
                        int rows, int cols) {
  copy2d_kernel<<<grid_for(ctx, (size_t)rows * cols), 256, 0, ctx->stream>>>(src, lds, dst, ldd,
                                                                             rows, cols);
  ctx->launches++;
  return la_check_launch(ctx, "copy2d_kernel");
}
