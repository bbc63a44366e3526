// Persistent triangular solves for a few right-hand sides (the correction
// solves of iterative refinement and the preconditioner of GMRES-IR).
//
// One launch per triangle. The matrix is cut into 64-row blocks; CTA t (in the
// order of an atomic ticket, so every block a CTA waits for belongs to a CTA
// that is already running) owns block b and computes
//   y_b = D_b^-1 (x_b - sum_{k before b} T_bk y_k)
// where D_b^-1 is the inverted diagonal block (computed once per factorization
// by invert_diag_kernel). It takes each earlier block as soon as that block's
// flag is published (release/acquire), so the solve proceeds as a wavefront
// whose critical path per block is one 64x64 block product, not a 64-step
// chain. Forward (unit L) runs blocks top-down, backward (U) bottom-up.
// Every wait is bounded (2 s); a CTA that gives up records an error and
// returns without publishing, which releases its dependants the same way.
#include "la_internal.cuh"

namespace {

constexpr int BS = 64;
constexpr int TT = 256;
constexpr int MAXR = 16;
constexpr unsigned long long WAIT_NS = 2000000000ull;

__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Inverse of each diagonal block: which = 0 for unit-lower L, 1 for upper U.
// One CTA per (block, which); thread j computes column j of the inverse, in
// the vector precision T from factors of precision TF.
template <typename TF, typename T>
__global__ void invert_diag_kernel(const TF* __restrict__ LU, size_t ld, int n, T* __restrict__ dinv) {
  extern __shared__ __align__(16) double inv_smem[];
  T(*a)[BS + 1] = reinterpret_cast<T(*)[BS + 1]>(inv_smem);
  T(*x)[BS + 1] = reinterpret_cast<T(*)[BS + 1]>(reinterpret_cast<T*>(inv_smem) + BS * (BS + 1));
  const int b = blockIdx.x, which = blockIdx.y;
  const int r0 = b * BS, bs = min(BS, n - r0);
  for (int idx = threadIdx.x; idx < BS * BS; idx += blockDim.x) {
    int i = idx / BS, k = idx % BS;
    a[i][k] = (i < bs && k < bs) ? (T)LU[(size_t)(r0 + i) * ld + r0 + k] : T(0);
  }
  __syncthreads();
  const int j = threadIdx.x;
  if (j < BS) {
    if (which == 0) {
      for (int i = 0; i < BS; i++) {
        T s = (i == j) ? T(1) : T(0);
        for (int k = j; k < i; k++) s = fma(-a[i][k], x[k][j], s);
        x[i][j] = (i < bs) ? s : T(0);
      }
    } else {
      for (int i = BS - 1; i >= 0; i--) {
        if (i >= bs) { x[i][j] = T(0); continue; }
        T s = (i == j) ? T(1) : T(0);
        for (int k = i + 1; k < bs; k++) s = fma(-a[i][k], x[k][j], s);
        x[i][j] = s / a[i][i];
      }
    }
  }
  __syncthreads();
  T* out = dinv + ((size_t)b * 2 + which) * BS * BS;
  for (int idx = threadIdx.x; idx < BS * BS; idx += blockDim.x) out[idx] = x[idx / BS][idx % BS];
}

// Factors in TF (FP32 for the mixed LU), vectors and the inverted diagonal
// blocks in T (FP64 for GMRES-IR, whose preconditioner must run at working
// precision; FP32 for plain refinement).
constexpr int LPRE = BS * BS / TT;    // elements of an off-diagonal tile per thread
constexpr int YPRE = BS * MAXR / TT;  // elements of a block of x per thread

template <typename TF, typename T>
constexpr size_t wave_smem() {
  return sizeof(T) * (BS * (BS + 1) + 3 * BS * MAXR) + sizeof(TF) * 2 * BS * (BS + 1);
}

// Largest u' >= u whose block is already solved, looking at most 8 blocks
// further (a solved block implies every earlier one is solved).
__device__ __forceinline__ int peek_solved(const int* flags, int nb, bool upper, int u, int t) {
  const int lim = min(t - 1, u + 8);
  while (u < lim) {
    const int kb = upper ? nb - 2 - u : u + 1;
    if (ld_acquire(flags + kb) == 0) break;
    u++;
  }
  return u;
}

// CTA with ticket t owns block b and takes the t earlier blocks in order
// (u = 0 .. t-1). The history loop is pipelined: the next off-diagonal tile is
// loaded into registers while the current one is applied, and the next block
// of x too once its flag is known to be set, so a CTA that is far from the
// frontier applies a block per tile product instead of per two memory round
// trips. The terms of each element are applied in the same order as a plain
// loop over u and k.
template <typename TF, typename T, bool UPPER>
__global__ void __launch_bounds__(TT)
trsv_wave_kernel(const TF* __restrict__ LU, size_t ld, const T* __restrict__ dinv, T* X, size_t ldx,
                 int n, int nrhs, int nb, int* flags, int* ticket, int* err) {
  extern __shared__ __align__(16) double wave_raw[];
  T(*db)[BS + 1] = reinterpret_cast<T(*)[BS + 1]>(wave_raw);
  T(*ys)[BS][MAXR] = reinterpret_cast<T(*)[BS][MAXR]>(reinterpret_cast<T*>(wave_raw) +
                                                      BS * (BS + 1));
  T(*acc)[MAXR] = reinterpret_cast<T(*)[MAXR]>(reinterpret_cast<T*>(wave_raw) + BS * (BS + 1) +
                                               2 * BS * MAXR);
  TF(*lb)[BS][BS + 1] = reinterpret_cast<TF(*)[BS][BS + 1]>(reinterpret_cast<T*>(wave_raw) +
                                                            BS * (BS + 1) + 3 * BS * MAXR);
  __shared__ int s_t;
  __shared__ int s_known;
  __shared__ int s_ok;
  const int tid = threadIdx.x;
  if (tid == 0) s_t = atomicAdd(ticket, 1);
  __syncthreads();
  const int t = s_t;
  const int b = UPPER ? nb - 1 - t : t;
  const int r0 = b * BS, bs = min(BS, n - r0);
  const int i = tid >> 2, jq = tid & 3;  // row of the block, first of 4 rhs columns

  for (int idx = tid; idx < BS * MAXR; idx += TT) {
    int r = idx / MAXR, c = idx % MAXR;
    acc[r][c] = (r < bs && c < nrhs) ? X[(size_t)(r0 + r) * ldx + c] : T(0);
  }
  {
    const T* d = dinv + ((size_t)b * 2 + (UPPER ? 1 : 0)) * BS * BS;
    for (int idx = tid; idx < BS * BS; idx += TT) db[idx / BS][idx % BS] = __ldg(d + idx);
  }

  TF pre[LPRE];
  T yv[YPRE];
  auto fetch_tile = [&](int u) {
    const int kb = UPPER ? nb - 1 - u : u;
    const int k0 = kb * BS, kbs = min(BS, n - k0);
#pragma unroll
    for (int e = 0; e < LPRE; e++) {
      const int idx = tid + TT * e;
      const int r = idx / BS, k = idx % BS;
      pre[e] = (r < bs && k < kbs) ? __ldg(LU + (size_t)(r0 + r) * ld + k0 + k) : TF(0);
    }
  };
  auto fetch_x = [&](int u, T (&dst)[YPRE]) {
    const int kb = UPPER ? nb - 1 - u : u;
    const int k0 = kb * BS, kbs = min(BS, n - k0);
#pragma unroll
    for (int e = 0; e < YPRE; e++) {
      const int idx = tid + TT * e;
      const int r = idx / MAXR, c = idx % MAXR;
      dst[e] = (r < kbs && c < nrhs) ? __ldcg(X + (size_t)(k0 + r) * ldx + c) : T(0);
    }
  };

  int known = -1;       // last block u known to be solved (uniform)
  bool have_y = false;  // yv holds block u's x (uniform)
  if (t > 0) fetch_tile(0);
  for (int u = 0; u < t; u++) {
    const int buf = u & 1;
#pragma unroll
    for (int e = 0; e < LPRE; e++) {
      const int idx = tid + TT * e;
      lb[buf][idx / BS][idx % BS] = pre[e];
    }
    if (have_y) {
#pragma unroll
      for (int e = 0; e < YPRE; e++) {
        const int idx = tid + TT * e;
        ys[buf][idx / MAXR][idx % MAXR] = yv[e];
      }
    }
    if (u + 1 < t) fetch_tile(u + 1);
    if (!have_y) {
      if (tid == 0) {
        int ok = 1;
        int kn = known;
        if (kn < u) {
          const int kb = UPPER ? nb - 1 - u : u;
          unsigned long long t0 = 0;
          unsigned spins = 0;
          while (ld_acquire(flags + kb) == 0) {
            if ((++spins & 63u) == 0) {
              if (*reinterpret_cast<volatile int*>(err) != 0) { ok = 0; break; }
              unsigned long long now = gtime();
              if (t0 == 0) t0 = now;
              else if (now - t0 > WAIT_NS) { atomicCAS(err, 0, (int)DERR_TRSV_TIMEOUT); ok = 0; break; }
            }
          }
          if (ok) kn = peek_solved(flags, nb, UPPER, u, t);
        }
        s_known = kn;
        s_ok = ok;
      }
      __syncthreads();
      if (!s_ok) return;
      known = s_known;
      T yt[YPRE];
      fetch_x(u, yt);
#pragma unroll
      for (int e = 0; e < YPRE; e++) {
        const int idx = tid + TT * e;
        ys[buf][idx / MAXR][idx % MAXR] = yt[e];
      }
    }
    have_y = (u + 1 < t) && known >= u + 1;
    if (have_y) fetch_x(u + 1, yv);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < MAXR / 4; q++) {
      const int j = jq + 4 * q;
      if (j < nrhs) {
        T s = acc[i][j];
        for (int k = 0; k < BS; k++) s = fma(-(T)lb[buf][i][k], ys[buf][k][j], s);
        acc[i][j] = s;
      }
    }
  }
  __syncthreads();
  // y_b = D_b^-1 acc
#pragma unroll
  for (int q = 0; q < MAXR / 4; q++) {
    const int j = jq + 4 * q;
    if (j < nrhs && i < bs) {
      T s = T(0);
      for (int k = 0; k < BS; k++) s = fma(db[i][k], acc[k][j], s);
      X[(size_t)(r0 + i) * ldx + j] = s;
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) st_release(flags + b, 1);
}

}  // namespace

cudaError_t configure_wave() {
  static la_device_once once;
  return once.run([](int) {
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(invert_diag_kernel<float, double>, at,
                                         (int)(2 * BS * (BS + 1) * sizeof(double)));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(invert_diag_kernel<float, float>, at,
                               (int)(2 * BS * (BS + 1) * sizeof(float)));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(trsv_wave_kernel<float, double, false>, at,
                               (int)wave_smem<float, double>());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(trsv_wave_kernel<float, double, true>, at,
                               (int)wave_smem<float, double>());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(trsv_wave_kernel<float, float, false>, at,
                               (int)wave_smem<float, float>());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(trsv_wave_kernel<float, float, true>, at,
                               (int)wave_smem<float, float>());
    return e;
  });
}

la_status launch_invert_diag_f32(la_ctx ctx, const float* LU, size_t ld, int n, double* dinv) {
  const int nb = (n + BS - 1) / BS;
  LA_CUDA(ctx, configure_wave());
  invert_diag_kernel<float, double><<<dim3(nb, 2), BS, 2 * BS * (BS + 1) * sizeof(double),
                                      ctx->stream>>>(LU, ld, n, dinv);
  ctx->launches++;
  return la_check_launch(ctx, "invert_diag_kernel");
}

// X (n x nrhs FP64, pitch ldx) <- U^-1 L^-1 X with unit-lower L and upper U
// packed in the FP32 LU; dinv (FP64) from launch_invert_diag_f32. `sync` is
// device scratch of at least 2 * (nb + 1) ints.
la_status launch_trsv_wave_f32(la_ctx ctx, const float* LU, size_t ld, const double* dinv,
                               double* X, size_t ldx, int n, int nrhs, int* sync) {
  if (nrhs > MAXR) return LA_UNSUPPORTED;
  const int nb = (n + BS - 1) / BS;
  int* fl = sync;
  int* fu = sync + nb;
  int* tickets = sync + 2 * nb;
  LA_CUDA(ctx, cudaMemsetAsync(sync, 0, (2 * nb + 2) * sizeof(int), ctx->stream));
  LA_CUDA(ctx, configure_wave());
  const size_t sm = wave_smem<float, double>();
  trsv_wave_kernel<float, double, false><<<nb, TT, sm, ctx->stream>>>(LU, ld, dinv, X, ldx, n, nrhs,
                                                                     nb, fl, tickets, ctx->d_err);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "trsv_wave_kernel"));
  trsv_wave_kernel<float, double, true><<<nb, TT, sm, ctx->stream>>>(LU, ld, dinv, X, ldx, n, nrhs,
                                                                    nb, fu, tickets + 1, ctx->d_err);
  ctx->launches++;
  return la_check_launch(ctx, "trsv_wave_kernel");
}

// FP32 vectors (the correction solves of plain refinement, which only need
// the factorization's own accuracy): inverted blocks in FP32 too.
la_status launch_invert_diag_f32f(la_ctx ctx, const float* LU, size_t ld, int n, float* dinv) {
  const int nb = (n + BS - 1) / BS;
  LA_CUDA(ctx, configure_wave());
  invert_diag_kernel<float, float><<<dim3(nb, 2), BS, 2 * BS * (BS + 1) * sizeof(float),
                                     ctx->stream>>>(LU, ld, n, dinv);
  ctx->launches++;
  return la_check_launch(ctx, "invert_diag_kernel");
}

la_status launch_trsv_wave_f32f(la_ctx ctx, const float* LU, size_t ld, const float* dinv,
                                float* X, size_t ldx, int n, int nrhs, int* sync) {
  if (nrhs > MAXR) return LA_UNSUPPORTED;
  const int nb = (n + BS - 1) / BS;
  int* fl = sync;
  int* fu = sync + nb;
  int* tickets = sync + 2 * nb;
  LA_CUDA(ctx, cudaMemsetAsync(sync, 0, (2 * nb + 2) * sizeof(int), ctx->stream));
  LA_CUDA(ctx, configure_wave());
  const size_t sm = wave_smem<float, float>();
  trsv_wave_kernel<float, float, false><<<nb, TT, sm, ctx->stream>>>(LU, ld, dinv, X, ldx, n, nrhs,
                                                                    nb, fl, tickets, ctx->d_err);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "trsv_wave_kernel"));
  trsv_wave_kernel<float, float, true><<<nb, TT, sm, ctx->stream>>>(LU, ld, dinv, X, ldx, n, nrhs,
                                                                   nb, fu, tickets + 1, ctx->d_err);
  ctx->launches++;
  return la_check_launch(ctx, "trsv_wave_kernel");
}
