// FP64 GEMM tiles for the blocked LU (trailing update, triangular-solve
// updates) and for Matrix * Matrix.
//
// GB300 executes FP64 FMA at roughly 2 per clock per SM (about 1.2 TFLOP/s for
// the chip), two orders of magnitude below its tensor rates, so these tiles are
// bound by the FP64 pipe, not by memory: a 64x64 output tile with a 32-deep K
// slab needs 32 KB of operands for 131k FMAs. The kernel therefore aims at
// keeping every SM's FP64 pipe fed (several resident CTAs, register-blocked
// 4x4 micro-tiles, cp.async double buffering) rather than at operand reuse.
//
// The FMA modes of the FP64 tiles with N > 16 (the LU's trailing update and
// Matrix * Matrix) stage their operand slabs with TMA (gemm_f64_tma_kernel):
// thread 0 issues two-dimensional tiled copies of the next A and B slabs into
// the other half of a two-stage ring while all threads compute on the current
// one, and the copies complete on an mbarrier. The other modes, narrow N and
// operands that break TMA's 16-byte alignment rules use cp.async
// (gemm_f64_kernel).
//
// Each output element is accumulated by one thread in a fixed k order, which
// gives the EXACT modes the reference's summation order: src/matrix/mod.rs:
// 965-973 (Mul: res = res + a*b from zero, ascending idx) and src/decomp/lu.rs:
// 124-126 (s = s + l*u, ascending k) and :260/:272 (x = x - x_k*l, per term).
#include "la_internal.cuh"
#include "tma_util.cuh"

namespace {

constexpr int BM = 64;
constexpr int BK = 32;
constexpr int THREADS = 256;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, int src_bytes) {
  unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem),
               "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::); }

// Loads one K slab: A rows [m0, m0+64) x k [k0, k0+32) and B k [k0, k0+32) x cols [n0, n0+BN)
// in 16-byte chunks (EPC elements). Out-of-range parts of a chunk are
// zero-filled by cp.async's source size, never read.
template <typename T, int BN>
__device__ __forceinline__ void load_slab(T* As, T* Bs, const T* A, size_t lda, const T* B,
                                          size_t ldb, int M, int N, int K, int m0, int n0,
                                          int k0) {
  constexpr int EPC = 16 / sizeof(T);
  const int tid = threadIdx.x;
  constexpr int ACH = BM * BK / EPC;
#pragma unroll
  for (int t = 0; t < ACH / THREADS; t++) {
    int chunk = tid + t * THREADS;
    int r = chunk / (BK / EPC);
    int kc = (chunk % (BK / EPC)) * EPC;
    int gr = m0 + r, gk = k0 + kc;
    int bytes = 0;
    const T* src = A;
    if (gr < M && gk < K) {
      bytes = min(EPC, K - gk) * (int)sizeof(T);
      src = A + (size_t)gr * lda + gk;
    }
    cp_async16(As + r * BK + kc, src, bytes);
  }
  constexpr int BCH = BK * BN / EPC;
#pragma unroll
  for (int t = 0; t < (BCH + THREADS - 1) / THREADS; t++) {
    int chunk = tid + t * THREADS;
    if (chunk < BCH) {
      int kr = chunk / (BN / EPC);
      int cc = (chunk % (BN / EPC)) * EPC;
      int gk = k0 + kr, gc = n0 + cc;
      int bytes = 0;
      const T* src = B;
      if (gk < K && gc < N) {
        bytes = min(EPC, N - gc) * (int)sizeof(T);
        src = B + (size_t)gk * ldb + gc;
      }
      cp_async16(Bs + kr * BN + cc, src, bytes);
    }
  }
}

// 256 threads; thread (tx = tid % 16, ty = tid / 16) owns rows ty + 16*i (i < 4)
// and cols tx + 16*j (j < BN/16) of the 64 x BN output tile.
template <typename T, int MODE, int BN>
__global__ void __launch_bounds__(THREADS)
gemm_f64_kernel(int M, int N, int K, const T* __restrict__ A, size_t lda,
                const T* __restrict__ B, size_t ldb, T* __restrict__ C, size_t ldc, int kper,
                size_t czs) {
  la_pdl_wait();
  la_pdl_trigger();
  constexpr int TN = BN / 16;
  extern __shared__ __align__(16) double smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  T* As = smem;                 // [2][BM][BK]
  T* Bs = smem + 2 * BM * BK;   // [2][BK][BN]

  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  // split K: this CTA's k range [kb, ke) and its own output slice
  const int kb = blockIdx.z * kper, ke = min(K, kb + kper);
  C += blockIdx.z * czs;

  T acc[4][TN];
  constexpr bool ZERO = (MODE == GM_FMA_ZERO || MODE == GM_EXACT_ZERO);
  constexpr bool DESC = (MODE == GM_EXACT_SUB_DESC || MODE == GM_FMA_SUB_DESC);
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) {
      int r = m0 + ty + 16 * i, c = n0 + tx + 16 * j;
      acc[i][j] = (!ZERO && r < M && c < N) ? C[(size_t)r * ldc + c] : T(0);
    }

  const int nslab = (ke - kb + BK - 1) / BK;
  // Slab order: ascending, or descending for back substitution.
  auto slab_k0 = [&](int s) { return kb + (DESC ? (nslab - 1 - s) * BK : s * BK); };

  load_slab<T, BN>(As, Bs, A, lda, B, ldb, M, N, ke, m0, n0, slab_k0(0));
  cp_async_commit();

  for (int s = 0; s < nslab; s++) {
    const int buf = s & 1;
    if (s + 1 < nslab) {
      load_slab<T, BN>(As + (buf ^ 1) * BM * BK, Bs + (buf ^ 1) * BK * BN, A, lda, B, ldb, M, N,
                       ke, m0, n0, slab_k0(s + 1));
      cp_async_commit();
      cp_async_wait_1();
    } else {
      cp_async_wait_all();
    }
    __syncthreads();
    const T* as = As + buf * BM * BK;
    const T* bs = Bs + buf * BK * BN;
    const int k0 = slab_k0(s);
    const int kn = min(BK, ke - k0);
    if (kn == BK) {
#pragma unroll 8
      for (int kk = 0; kk < BK; kk++) {
        const int k = DESC ? (BK - 1 - kk) : kk;
        T a[4], b[TN];
#pragma unroll
        for (int i = 0; i < 4; i++) a[i] = as[(ty + 16 * i) * BK + k];
#pragma unroll
        for (int j = 0; j < TN; j++) b[j] = bs[k * BN + tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < TN; j++) {
            if (MODE == GM_FMA_SUB || MODE == GM_FMA_SUB_DESC)
              acc[i][j] = fma(-a[i], b[j], acc[i][j]);
            else if (MODE == GM_FMA_ZERO)
              acc[i][j] = fma(a[i], b[j], acc[i][j]);
            else if (MODE == GM_EXACT_ADD || MODE == GM_EXACT_ZERO)
              acc[i][j] = __dadd_rn(acc[i][j], __dmul_rn(a[i], b[j]));
            else
              acc[i][j] = __dsub_rn(acc[i][j], __dmul_rn(a[i], b[j]));
          }
      }
    } else {
      // Ragged last slab: only the kn valid k are applied (no padded terms).
      for (int kk = 0; kk < kn; kk++) {
        const int k = DESC ? (kn - 1 - kk) : kk;
        T a[4], b[TN];
#pragma unroll
        for (int i = 0; i < 4; i++) a[i] = as[(ty + 16 * i) * BK + k];
#pragma unroll
        for (int j = 0; j < TN; j++) b[j] = bs[k * BN + tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
          for (int j = 0; j < TN; j++) {
            if (MODE == GM_FMA_SUB || MODE == GM_FMA_SUB_DESC)
              acc[i][j] = fma(-a[i], b[j], acc[i][j]);
            else if (MODE == GM_FMA_ZERO)
              acc[i][j] = fma(a[i], b[j], acc[i][j]);
            else if (MODE == GM_EXACT_ADD || MODE == GM_EXACT_ZERO)
              acc[i][j] = __dadd_rn(acc[i][j], __dmul_rn(a[i], b[j]));
            else
              acc[i][j] = __dsub_rn(acc[i][j], __dmul_rn(a[i], b[j]));
          }
      }
    }
    __syncthreads();
  }

#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) {
      int r = m0 + ty + 16 * i, c = n0 + tx + 16 * j;
      if (r < M && c < N) C[(size_t)r * ldc + c] = acc[i][j];
    }
}

// TMA-staged FP64 tile (FMA modes): 64 x 64 output tile per 256-thread CTA,
// 32-deep K slabs in a two-stage ring. A slab of A is one TMA box of 64 rows x
// 32 columns (dense [64][32]); a slab of B is two boxes of 32 k-rows x 32
// columns (dense [2][32][32]), keeping every box row at 256 bytes. Zero fill
// covers the matrix edges; the last slab applies only its valid k. Each wait
// is bounded: a CTA that gives up records DERR_GEMM_TIMEOUT, drains its own
// copies (bounded) and exits with every thread, without writing C.
constexpr int TMA_BN = 64;
constexpr int TMA_STAGE_D = BM * BK + BK * TMA_BN;  // doubles per stage
constexpr uint32_t TMA_STAGE_BYTES = TMA_STAGE_D * sizeof(double);
constexpr size_t TMA_SMEM = 2 * (size_t)TMA_STAGE_BYTES + 1024;  // + alignment slack

template <int MODE>
__global__ void __launch_bounds__(THREADS)
gemm_f64_tma_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
                    int M, int N, int K, double* __restrict__ C, size_t ldc, int* err, int kper,
                    size_t czs, int tri) {
  extern __shared__ __align__(1024) unsigned char tma_raw[];
  __shared__ __align__(8) uint64_t full[2];
  double* smem = reinterpret_cast<double*>(
      (reinterpret_cast<uintptr_t>(tma_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  int by = blockIdx.y, bx = blockIdx.x;
  if (tri) {  // lower-triangular tile grid: blockIdx.x enumerates (by, bx), bx <= by, row-major
    const int t = blockIdx.x;
    int r = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((r + 1) * (r + 2) / 2 <= t) r++;
    while (r * (r + 1) / 2 > t) r--;
    by = r;
    bx = t - r * (r + 1) / 2;
  }
  const int m0 = by * BM, n0 = bx * TMA_BN;
  constexpr bool ZERO = MODE == GM_FMA_ZERO;
  const int kb = blockIdx.z * kper, ke = min(K, kb + kper);  // split K
  C += blockIdx.z * czs;

  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int r = m0 + ty + 16 * i, c = n0 + tx + 16 * j;
      acc[i][j] = (!ZERO && r < M && c < N) ? C[(size_t)r * ldc + c] : 0.0;
    }

  const int nslab = (ke - kb + BK - 1) / BK;
  if (tid == 0) {
    la_tma::mbar_init(&full[0], 1);
    la_tma::mbar_init(&full[1], 1);
    la_tma::mbar_init_fence();
  }
  __syncthreads();
  auto issue = [&](int stage, int s) {
    double* st = smem + stage * TMA_STAGE_D;
    la_tma::mbar_expect_tx(&full[stage], TMA_STAGE_BYTES);
    la_tma::tma_load_2d(st, &ta, kb + s * BK, m0, &full[stage]);
    la_tma::tma_load_2d(st + BM * BK, &tb, n0, kb + s * BK, &full[stage]);
    la_tma::tma_load_2d(st + BM * BK + BK * 32, &tb, n0 + 32, kb + s * BK, &full[stage]);
  };
  if (tid == 0 && nslab > 0) issue(0, 0);

  for (int s = 0; s < nslab; s++) {
    const int buf = s & 1;
    if (tid == 0 && s + 1 < nslab) issue(buf ^ 1, s + 1);
    const bool ok =
        la_tma::mbar_wait(&full[buf], (uint32_t)((s >> 1) & 1), err, (int)DERR_GEMM_TIMEOUT);
    const double* as = smem + buf * TMA_STAGE_D;
    const double* bs = as + BM * BK;
    const int kn = min(BK, ke - kb - s * BK);
    if (ok) {
#pragma unroll 8
      for (int k = 0; k < BK; k++) {
        if (k < kn) {
          double a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; i++) a[i] = as[(ty + 16 * i) * BK + k];
#pragma unroll
          for (int j = 0; j < 4; j++) b[j] = bs[(j >> 1) * BK * 32 + k * 32 + tx + 16 * (j & 1)];
#pragma unroll
          for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++)
              acc[i][j] = ZERO ? fma(a[i], b[j], acc[i][j]) : fma(-a[i], b[j], acc[i][j]);
        }
      }
    }
    if (__syncthreads_or(!ok)) {
      // Give up: drain this CTA's copies still in flight, then every thread exits.
      if (tid == 0) {
        la_tma::mbar_drain(&full[buf], (uint32_t)((s >> 1) & 1));
        if (s + 1 < nslab) la_tma::mbar_drain(&full[buf ^ 1], (uint32_t)(((s + 1) >> 1) & 1));
      }
      return;
    }
  }

#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int r = m0 + ty + 16 * i, c = n0 + tx + 16 * j;
      if (r < M && c < N) C[(size_t)r * ldc + c] = acc[i][j];
    }
}

constexpr size_t GEMM_SMEM_CAP = 96 * 1024;

// The TMA form of the FMA modes; LA_UNSUPPORTED (nothing launched) when an
// operand breaks TMA's rules (16-byte aligned bases, pitches of whole 16-byte
// units) so that the caller uses the cp.async form.
template <int MODE>
la_status launch_tma(la_ctx ctx, int M, int N, int K, const double* A, size_t lda,
                     const double* B, size_t ldb, double* C, size_t ldc, size_t min_smem,
                     int splits = 1, int kper = 0, size_t czs = 0, bool tri = false) {
  if (K <= 0 || (reinterpret_cast<uintptr_t>(A) % 16) || (reinterpret_cast<uintptr_t>(B) % 16) ||
      (lda % 2) || (ldb % 2))
    return LA_UNSUPPORTED;
  CUtensorMap ta, tb;
  if (!la_tma::encode_2d(ctx, &ta, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, A, (size_t)M, (size_t)K,
                         lda, (uint32_t)BK, (uint32_t)BM, CU_TENSOR_MAP_SWIZZLE_NONE) ||
      !la_tma::encode_2d(ctx, &tb, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, B, (size_t)K, (size_t)N,
                         ldb, 32u, (uint32_t)BK, CU_TENSOR_MAP_SWIZZLE_NONE))
    return LA_UNSUPPORTED;
  static la_device_once configured;  // one attribute call per instantiation and device
  cudaError_t e = configured.run([](int) {
    return cudaFuncSetAttribute(gemm_f64_tma_kernel<MODE>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GEMM_SMEM_CAP);
  });
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaFuncSetAttribute(gemm_tma)");
  const size_t smem = std::min(GEMM_SMEM_CAP, std::max(TMA_SMEM, min_smem));
  const int tm = (M + BM - 1) / BM;
  dim3 grid(tri ? tm * (tm + 1) / 2 : (N + TMA_BN - 1) / TMA_BN, tri ? 1 : tm, splits);
  gemm_f64_tma_kernel<MODE><<<grid, THREADS, smem, ctx->stream>>>(
      ta, tb, M, N, K, C, ldc, ctx->d_err, splits > 1 ? kper : K, czs, tri ? 1 : 0);
  ctx->launches++;
  return la_check_launch(ctx, "gemm_f64_tma_kernel");
}

template <int MODE, int BN, typename T = double>
la_status launch_mode(la_ctx ctx, int M, int N, int K, const T* A, size_t lda, const T* B,
                      size_t ldb, T* C, size_t ldc, size_t min_smem, int splits = 1,
                      int kper = 0, size_t czs = 0) {
  const size_t smem =
      std::min(GEMM_SMEM_CAP, std::max((size_t)2 * (BM * BK + BK * BN) * sizeof(T), min_smem));
  static la_device_once configured;  // one attribute call per instantiation and device
  cudaError_t e = configured.run([](int) {
    return cudaFuncSetAttribute(gemm_f64_kernel<T, MODE, BN>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GEMM_SMEM_CAP);
  });
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaFuncSetAttribute(gemm)");
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, splits);
  e = la_launch(ctx, gemm_f64_kernel<T, MODE, BN>, grid, dim3(THREADS), smem, ctx->stream, M, N, K,
                A, lda, B, ldb, C, ldc, splits > 1 ? kper : K, czs);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "gemm_f64_kernel launch");
  ctx->launches++;
  return la_check_launch(ctx, "gemm_f64_kernel");
}

template <int BN>
la_status launch_bn(la_ctx ctx, int mode, int M, int N, int K, const double* A, size_t lda,
                    const double* B, size_t ldb, double* C, size_t ldc, size_t ms) {
  switch (mode) {
    case GM_FMA_SUB: return launch_mode<GM_FMA_SUB, BN>(ctx, M, N, K, A, lda, B, ldb, C, ldc, ms);
    case GM_FMA_ZERO: return launch_mode<GM_FMA_ZERO, BN>(ctx, M, N, K, A, lda, B, ldb, C, ldc, ms);
    case GM_EXACT_ADD: return launch_mode<GM_EXACT_ADD, BN>(ctx, M, N, K, A, lda, B, ldb, C, ldc, ms);
    case GM_EXACT_ZERO: return launch_mode<GM_EXACT_ZERO, BN>(ctx, M, N, K, A, lda, B, ldb, C, ldc, ms);
    case GM_EXACT_SUB: return launch_mode<GM_EXACT_SUB, BN>(ctx, M, N, K, A, lda, B, ldb, C, ldc, ms);
    case GM_EXACT_SUB_DESC:
      return launch_mode<GM_EXACT_SUB_DESC, BN>(ctx, M, N, K, A, lda, B, ldb, C, ldc, ms);
    case GM_FMA_SUB_DESC:
      return launch_mode<GM_FMA_SUB_DESC, BN>(ctx, M, N, K, A, lda, B, ldb, C, ldc, ms);
    default: return LA_INVALID;
  }
}

}  // namespace

// C (M x N, ldc) op= A (M x K, lda) * B (K x N, ldb); all row-major. Pointers
// must be 16-byte aligned and pitches even (the library pads pitches to 4).
la_status launch_gemm(la_ctx ctx, int mode, int M, int N, int K, const double* A, size_t lda,
                      const double* B, size_t ldb, double* C, size_t ldc, size_t min_smem) {
  if (M <= 0 || N <= 0) return LA_OK;
  if (K <= 0 && mode != GM_FMA_ZERO && mode != GM_EXACT_ZERO) return LA_OK;
  if (N <= 16) return launch_bn<16>(ctx, mode, M, N, K, A, lda, B, ldb, C, ldc, min_smem);
  if (mode == GM_FMA_SUB || mode == GM_FMA_ZERO) {
    const la_status s =
        mode == GM_FMA_SUB
            ? launch_tma<GM_FMA_SUB>(ctx, M, N, K, A, lda, B, ldb, C, ldc, min_smem)
            : launch_tma<GM_FMA_ZERO>(ctx, M, N, K, A, lda, B, ldb, C, ldc, min_smem);
    if (s != LA_UNSUPPORTED) return s;
  }
  return launch_bn<64>(ctx, mode, M, N, K, A, lda, B, ldb, C, ldc, min_smem);
}

// Split-K product for tall-skinny inner products (C = A B with K >> M): the
// K range is cut into `splits` pieces of kper (a multiple of the 32-deep slab),
// and piece z writes its own partial product C + z * czs (z < splits), which
// the caller sums. Fused arithmetic from zero, as GM_FMA_ZERO.
la_status launch_gemm_splitk(la_ctx ctx, int M, int N, int K, const double* A, size_t lda,
                             const double* B, size_t ldb, double* C, size_t ldc, size_t czs,
                             int splits, int kper) {
  if (M <= 0 || N <= 0) return LA_OK;
  if (splits < 1 || kper % BK != 0 || (size_t)(splits - 1) * kper >= (size_t)std::max(K, 1) ||
      (size_t)splits * kper < (size_t)K)
    return LA_INVALID;
  if (N > 16) {
    const la_status s =
        launch_tma<GM_FMA_ZERO>(ctx, M, N, K, A, lda, B, ldb, C, ldc, 0, splits, kper, czs);
    if (s != LA_UNSUPPORTED) return s;
    return launch_mode<GM_FMA_ZERO, 64>(ctx, M, N, K, A, lda, B, ldb, C, ldc, 0, splits, kper,
                                        czs);
  }
  return launch_mode<GM_FMA_ZERO, 16>(ctx, M, N, K, A, lda, B, ldb, C, ldc, 0, splits, kper, czs);
}

// C -= A B on the output tiles at or below the diagonal of the square C
// (M x M; 64 x 64 tiles, a diagonal tile in full): the symmetric trailing
// update of the Cholesky factorization. LA_UNSUPPORTED (nothing launched)
// where the TMA form cannot take the operands.
la_status launch_gemm_lower(la_ctx ctx, int M, int K, const double* A, size_t lda,
                            const double* B, size_t ldb, double* C, size_t ldc) {
  if (M <= 0 || K <= 0) return LA_OK;
  return launch_tma<GM_FMA_SUB>(ctx, M, M, K, A, lda, B, ldb, C, ldc, 0, 1, 0, 0, true);
}

// FP32 form (FAST arithmetic only) for the panels and triangular updates of the
// mixed-precision LU. Pointers 16-byte aligned, pitches multiples of 4.
la_status launch_gemm_f32(la_ctx ctx, int mode, int M, int N, int K, const float* A, size_t lda,
                          const float* B, size_t ldb, float* C, size_t ldc) {
  if (M <= 0 || N <= 0 || K <= 0) return LA_OK;
  if (mode != GM_FMA_SUB) return LA_INVALID;
  if (N <= 16) return launch_mode<GM_FMA_SUB, 16, float>(ctx, M, N, K, A, lda, B, ldb, C, ldc, 0);
  return launch_mode<GM_FMA_SUB, 64, float>(ctx, M, N, K, A, lda, B, ldb, C, ldc, 0);
}
