// Triangular solves of LUDecomposition::solve (src/decomp/lu.rs:256-275).
//
// Two schedules that apply every term in the same order, so their results are
// bit-identical:
//
// Wavefront (default). One persistent launch per triangle. The rows are cut
// into 32-row blocks and the right-hand sides into groups of 4 columns; a work
// item is (row block, column group), taken by CTAs from an atomic ticket in
// dependency order (forward: top block first; backward: bottom block first),
// so every item a CTA waits for belongs to a CTA that is already running. The
// item's 4 warps hold one column each, lane = row, in registers. For every
// finished block k (in the reference's order) it loads the 32 x 32 tile of
// L (or U) against k into shared memory (prefetched in registers a step
// ahead, since it does not depend on k being finished), waits until the
// column group's progress counter says block k is solved (acquire loads,
// bounded), reads x_k and applies the 32 terms; then it solves its diagonal
// block lane by lane with shuffles, stores x and publishes (release). The
// critical path per block is one tile application and one 32-step diagonal
// solve; the rest of the update work fills the other SMs.
//
// Block steps. One launch per 16-row block step: for the finished block
// [k0, k1),
//   tile 0    : rows of the next block [k1, k2): take the terms of block
//               [k0, k1), then solve the diagonal block (16 sequential steps)
//   tiles 1.. : rows [k2, n): take the terms of block [k0, k1)
// Backward (U, lu.rs:266-275) mirrors it from the bottom, with the division by
// u_kk when a row becomes final. grid.y splits the right-hand sides into
// 32-column chunks. Used for more than 4 * SOLVE_WAVE_MAX_GROUPS right-hand
// sides or when the wavefront is switched off.
//
// Order of the terms of row i (both schedules): forward (unit L, lu.rs:257-263)
// ascending k; backward (U, lu.rs:266-275) descending k, then the division by
// u_ii. EXACT applies each term as x_i = x_i - x_k * l_ik without fusion and
// divides; FAST uses FMA and multiplies by the reciprocal of u_ii (quot).
#include "la_internal.cuh"

namespace {

constexpr int SB = 16;    // block rows of the solve
constexpr int RT = 32;    // rows per update tile
constexpr int CT = 32;    // right-hand-side columns per CTA
constexpr int ST = 256;   // threads

template <bool EXACT, typename T>
__device__ __forceinline__ T apply(T x, T xk, T l) {
  if constexpr (EXACT) return __dsub_rn(x, __dmul_rn(xk, l));
  else return fma(-xk, l, x);
}

// A row's value over its diagonal entry d once its terms are in. EXACT: the
// division of the reference (lu.rs:272, cholesky.rs:127-139). FAST: the
// product with r = RN(1/d), taken before the row's turn, so no division sits
// on the solve's sequential chain (FP64 division is a long instruction
// sequence on this GPU's FP64 pipe); one extra rounding per row, far inside
// the FAST mode's backward-error bound. Both schedules use it, so their
// results stay bit-identical.
template <bool EXACT, typename T>
__device__ __forceinline__ T quot(T v, T d, T r) {
  if constexpr (EXACT) return v / d;
  else return v * r;
}

// UPPER = false: forward with unit L; UPPER = true: backward with U.
// kb_prev = size of the finished block at [k0, k0 + kb_prev) (0: no finished
// block, only solve the block that starts at `next0`).
template <typename T, bool EXACT, bool UPPER>
__global__ void __launch_bounds__(ST)
solve_step_kernel(const T* __restrict__ LU, size_t ld, T* __restrict__ X, size_t ldx,
                  int n, int nrhs, int k0, int kb_prev, int next0, int nextb) {
  __shared__ T xk[SB][CT];        // finished block's solution rows
  __shared__ T lt[RT][SB + 1];    // L/U entries of this tile against the finished block
  __shared__ T dg[SB][SB + 1];    // diagonal block (tile 0)
  __shared__ T xt[RT][CT];        // this tile's rows of X
  const int c0 = blockIdx.y * CT;
  const int tx = threadIdx.x % CT, ty = threadIdx.x / CT;  // ty 0..7
  const int col = c0 + tx;
  const bool colok = col < nrhs;
  const int tile = blockIdx.x;

  // Rows of this tile.
  int r0, rn;
  if (tile == 0) {
    r0 = next0;
    rn = nextb;
  } else if (!UPPER) {
    const int rest0 = next0 + nextb;
    r0 = rest0 + (tile - 1) * RT;
    rn = min(RT, n - r0);
  } else {
    // backward: rest rows are [0, next0), taken from the top
    r0 = (tile - 1) * RT;
    rn = min(RT, next0 - r0);
  }
  if (rn <= 0) return;

  if (kb_prev > 0) {
    for (int i = ty; i < kb_prev; i += ST / CT)
      xk[i][tx] = colok ? X[(size_t)(k0 + i) * ldx + col] : T(0);
    for (int idx = threadIdx.x; idx < rn * kb_prev; idx += ST) {
      const int i = idx / kb_prev, k = idx % kb_prev;
      lt[i][k] = LU[(size_t)(r0 + i) * ld + k0 + k];
    }
  }
  for (int i = ty; i < rn; i += ST / CT) xt[i][tx] = colok ? X[(size_t)(r0 + i) * ldx + col] : T(0);
  if (tile == 0) {
    for (int idx = threadIdx.x; idx < rn * rn; idx += ST) {
      const int i = idx / rn, k = idx % rn;
      dg[i][k] = LU[(size_t)(r0 + i) * ld + r0 + k];
    }
  }
  __syncthreads();

  // Terms of the finished block.
  if (kb_prev > 0) {
    for (int i = ty; i < rn; i += ST / CT) {
      T x = xt[i][tx];
      if (!UPPER) {
        for (int k = 0; k < kb_prev; k++) x = apply<EXACT, T>(x, xk[k][tx], lt[i][k]);
      } else {
        for (int k = kb_prev - 1; k >= 0; k--) x = apply<EXACT, T>(x, xk[k][tx], lt[i][k]);
      }
      xt[i][tx] = x;
    }
  }

  if (tile == 0) {
    __syncthreads();
    if (!UPPER) {
      for (int k = 0; k < rn; k++) {
        const T v = xt[k][tx];
        for (int i = ty; i < rn; i += ST / CT)
          if (i > k) xt[i][tx] = apply<EXACT, T>(xt[i][tx], v, dg[i][k]);
        __syncthreads();
      }
    } else {
      for (int k = rn - 1; k >= 0; k--) {
        if (ty == (k % (ST / CT))) xt[k][tx] = quot<EXACT>(xt[k][tx], dg[k][k], T(1) / dg[k][k]);
        __syncthreads();
        const T v = xt[k][tx];
        for (int i = ty; i < k; i += ST / CT) xt[i][tx] = apply<EXACT, T>(xt[i][tx], v, dg[i][k]);
        __syncthreads();
      }
    }
  }
  __syncthreads();
  if (colok)
    for (int i = ty; i < rn; i += ST / CT) X[(size_t)(r0 + i) * ldx + col] = xt[i][tx];
}

template <typename T, bool EXACT, bool UPPER>
la_status launch_step(la_ctx ctx, const T* LU, size_t ld, T* X, size_t ldx, int n,
                      int nrhs, int k0, int kb_prev, int next0, int nextb) {
  int rest;
  if (!UPPER) rest = n - (next0 + nextb);
  else rest = next0;
  if (kb_prev == 0) rest = 0;
  dim3 grid(1 + (rest + RT - 1) / RT, (nrhs + CT - 1) / CT);
  solve_step_kernel<T, EXACT, UPPER><<<grid, ST, 0, ctx->stream>>>(LU, ld, X, ldx, n, nrhs, k0,
                                                                   kb_prev, next0, nextb);
  ctx->launches++;
  return la_check_launch(ctx, "solve_step_kernel");
}

template <typename T, bool EXACT>
la_status solve_all(la_ctx ctx, const T* LU, size_t ld, T* X, size_t ldx, int n, int nrhs) {
  // Forward: block 0 alone, then one step per finished block.
  const int nb = (n + SB - 1) / SB;
  LA_TRY((launch_step<T, EXACT, false>(ctx, LU, ld, X, ldx, n, nrhs, 0, 0, 0, std::min(SB, n))));
  for (int b = 0; b + 1 < nb; b++) {
    const int k0 = b * SB, kb = std::min(SB, n - k0);
    const int nx0 = k0 + kb, nxb = std::min(SB, n - nx0);
    LA_TRY((launch_step<T, EXACT, false>(ctx, LU, ld, X, ldx, n, nrhs, k0, kb, nx0, nxb)));
  }
  // Backward: last block alone, then upward.
  const int last0 = (nb - 1) * SB;
  LA_TRY((launch_step<T, EXACT, true>(ctx, LU, ld, X, ldx, n, nrhs, 0, 0, last0, n - last0)));
  for (int b = nb - 1; b > 0; b--) {
    const int k0 = b * SB, kb = std::min(SB, n - k0);
    const int nx0 = (b - 1) * SB;
    LA_TRY((launch_step<T, EXACT, true>(ctx, LU, ld, X, ldx, n, nrhs, k0, kb, nx0, SB)));
  }
  return LA_OK;
}


// ---------------------------------------------------------------------------
// Wavefront schedule.

constexpr int WB = 32;                 // rows per block (one lane each)
constexpr int WC = 4;                  // right-hand-side columns per item (one warp each)
constexpr int WT = WB * WC;            // threads
constexpr int WPRE = WB * WB / WT;     // tile elements each thread prefetches
constexpr unsigned long long WAVE_WAIT_NS = 2000000000ull;

__device__ __forceinline__ unsigned long long wave_time() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int wave_ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void wave_st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// All 32 lanes of a warp wait until *p >= need; every lane's own acquire load
// saw the value, so each lane's later loads see the publisher's stores.
// Returns the smallest value the lanes saw, or -1 after an error elsewhere or
// 2 s without progress (then the error word holds DERR_TRSV_TIMEOUT).
__device__ __forceinline__ int wave_wait(const int* p, int need, int* err) {
  const unsigned full = 0xffffffffu;
  unsigned long long t0 = 0;
  unsigned spins = 0;
  for (;;) {
    const int v = wave_ld_acquire(p);
    if (__all_sync(full, v >= need)) return __reduce_min_sync(full, v);
    if ((++spins & 63u) == 0) {
      int bad = 0;
      if ((threadIdx.x & 31) == 0) {
        if (*reinterpret_cast<volatile int*>(err) != 0) {
          bad = 1;
        } else {
          const unsigned long long now = wave_time();
          if (t0 == 0) t0 = now;
          else if (now - t0 > WAVE_WAIT_NS) {
            atomicCAS(err, 0, (int)DERR_TRSV_TIMEOUT);
            bad = 1;
          }
        }
      }
      if (__shfl_sync(full, bad, 0)) return -1;
    }
  }
}

// Tile s of an item: s < q are the finished blocks in the reference's order,
// s = q the diagonal block. Both are rows [r0, r0 + sb) against the columns
// of block kb = UPPER ? nb - 1 - s : s.
template <typename T>
__device__ __forceinline__ void wave_fetch_tile(const T* __restrict__ LU, size_t ld, int n, int r0,
                                                int sb, int kb, T (&pre)[WPRE]) {
  const int k0 = kb * WB, kbs = min(WB, n - k0);
#pragma unroll
  for (int j = 0; j < WPRE; j++) {
    const int idx = threadIdx.x + WT * j;
    const int r = idx / WB, k = idx % WB;
    pre[j] = (r < sb && k < kbs) ? __ldg(LU + (size_t)(r0 + r) * ld + k0 + k) : T(0);
  }
}

// DIVL: the lower triangle has a non-unit diagonal (a Cholesky factor): each
// row's value is divided by it once its terms are applied.
template <typename T, bool EXACT, bool UPPER, bool DIVL = false>
__global__ void __launch_bounds__(WT)
solve_wave_kernel(const T* __restrict__ LU, size_t ld, T* X, size_t ldx, int n, int nrhs,
                  int nb, int groups, int* ticket, int* prog, int* err) {
  __shared__ T ls[2][WB][WB + 1];
  __shared__ int s_item;
  const unsigned full = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int items = nb * groups;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(ticket, 1);
    __syncthreads();
    const int t = s_item;
    if (t >= items) return;
    const int q = t / groups, g = t - q * groups;
    const int b = UPPER ? nb - 1 - q : q;
    const int r0 = b * WB, sb = min(WB, n - r0);
    const int col = g * WC + w;
    const bool colok = col < nrhs;  // warp-uniform
    int* pg = prog + g;

    T x = (lane < sb && colok) ? __ldcg(X + (size_t)(r0 + lane) * ldx + col) : T(0);
    T pre[WPRE];
    wave_fetch_tile<T>(LU, ld, n, r0, sb, UPPER ? nb - 1 : 0, pre);
    int known = 0;       // blocks of this column group known to be solved
    bool fail = false;   // warp-uniform
    T xn = T(0);         // x of the next finished block, when already fetched
    bool have_xn = false;
    for (int s = 0; s <= q; s++) {
      const int buf = s & 1;
      const int kb = UPPER ? nb - 1 - s : s;
      const int kbs = min(WB, n - kb * WB);
#pragma unroll
      for (int j = 0; j < WPRE; j++) {
        const int idx = tid + WT * j;
        ls[buf][idx / WB][idx % WB] = pre[j];
      }
      T xc = T(0);
      if (s < q && colok && !fail) {
        if (have_xn) {
          xc = xn;
        } else {
          if (known < s + 1) {
            const int v = wave_wait(pg, s + 1, err);
            if (v < 0) fail = true;
            else known = v;
          }
          if (!fail && lane < kbs) xc = __ldcg(X + (size_t)(kb * WB + lane) * ldx + col);
        }
      }
      if (s < q) wave_fetch_tile<T>(LU, ld, n, r0, sb, UPPER ? nb - 2 - s : s + 1, pre);
      have_xn = false;
      if (s + 1 < q && colok && !fail && known >= s + 2) {
        const int kn = UPPER ? nb - 2 - s : s + 1;
        xn = (lane < min(WB, n - kn * WB)) ? __ldcg(X + (size_t)(kn * WB + lane) * ldx + col)
                                           : T(0);
        have_xn = true;
      }
      __syncthreads();
      if (!colok || fail) continue;
      const T(*tile)[WB + 1] = ls[buf];
      if (s < q) {
        if (kbs == WB) {
          if (!UPPER) {
#pragma unroll
            for (int k = 0; k < WB; k++) x = apply<EXACT, T>(x, __shfl_sync(full, xc, k), tile[lane][k]);
          } else {
#pragma unroll
            for (int k = WB - 1; k >= 0; k--)
              x = apply<EXACT, T>(x, __shfl_sync(full, xc, k), tile[lane][k]);
          }
        } else {
          if (!UPPER) {
            for (int k = 0; k < kbs; k++) x = apply<EXACT, T>(x, __shfl_sync(full, xc, k), tile[lane][k]);
          } else {
            for (int k = kbs - 1; k >= 0; k--)
              x = apply<EXACT, T>(x, __shfl_sync(full, xc, k), tile[lane][k]);
          }
        }
      } else if (!UPPER && !DIVL) {
        for (int k = 0; k < sb; k++) {
          const T xk = __shfl_sync(full, x, k);
          if (lane > k) x = apply<EXACT, T>(x, xk, tile[lane][k]);
        }
      } else {
        // FAST: lane l takes the reciprocal of its row's diagonal entry once,
        // off the chain; EXACT divides on the chain as the reference does.
        const T rcp = (!EXACT && lane < sb) ? T(1) / tile[lane][lane] : T(1);
        if (!UPPER) {
          // as in the backward case: every lane divides row k's value in lockstep
          for (int k = 0; k < sb; k++) {
            const T xk = quot<EXACT>(__shfl_sync(full, x, k), tile[k][k], __shfl_sync(full, rcp, k));
            if (lane == k) x = xk;
            else if (lane > k) x = apply<EXACT, T>(x, xk, tile[lane][k]);
          }
        } else {
          // Every lane takes row k's undivided value and divides it by u_kk in
          // lockstep (the same operands give the same quotient in every lane),
          // so the division is not a divergent branch on the chain.
          for (int k = sb - 1; k >= 0; k--) {
            const T xk = quot<EXACT>(__shfl_sync(full, x, k), tile[k][k], __shfl_sync(full, rcp, k));
            if (lane == k) x = xk;
            else if (lane < k) x = apply<EXACT, T>(x, xk, tile[lane][k]);
          }
        }
      }
    }
    if (colok && !fail && lane < sb) X[(size_t)(r0 + lane) * ldx + col] = x;
    __threadfence();
    if (__syncthreads_or(fail ? 1 : 0)) return;
    if (tid == 0) wave_st_release(pg, q + 1);
  }
}

template <typename T, bool EXACT>
la_status solve_wave(la_ctx ctx, const T* LU, size_t ld, T* X, size_t ldx, int n, int nrhs) {
  const int nb = (n + WB - 1) / WB;
  const int groups = (nrhs + WC - 1) / WC;
  int* tickets = ctx->d_solve_sync;
  int* prog_l = tickets + 2;
  int* prog_u = prog_l + groups;
  LA_CUDA(ctx, cudaMemsetAsync(tickets, 0, (2 + 2 * (size_t)groups) * sizeof(int), ctx->stream));
  const long long items = (long long)nb * groups;
  const int grid = (int)std::min<long long>(items, (long long)ctx->solve_wave * ctx->sm_count);
  solve_wave_kernel<T, EXACT, false><<<grid, WT, 0, ctx->stream>>>(
      LU, ld, X, ldx, n, nrhs, nb, groups, tickets, prog_l, ctx->d_err);
  ctx->launches++;
  LA_TRY(la_check_launch(ctx, "solve_wave_kernel"));
  solve_wave_kernel<T, EXACT, true><<<grid, WT, 0, ctx->stream>>>(
      LU, ld, X, ldx, n, nrhs, nb, groups, tickets + 1, prog_u, ctx->d_err);
  ctx->launches++;
  return la_check_launch(ctx, "solve_wave_kernel");
}

// One triangle with the wavefront kernel, right-hand sides in chunks of at
// most 4 * SOLVE_WAVE_MAX_GROUPS columns.
template <bool EXACT, bool UPPER, bool DIVL>
la_status tri_wave(la_ctx ctx, const double* T, size_t ld, double* X, size_t ldx, int n,
                   int nrhs) {
  const int nb = (n + WB - 1) / WB;
  const int per = WC * SOLVE_WAVE_MAX_GROUPS;
  for (int c0 = 0; c0 < nrhs; c0 += per) {
    const int nr = std::min(per, nrhs - c0);
    const int groups = (nr + WC - 1) / WC;
    int* tickets = ctx->d_solve_sync;
    int* prog = tickets + 2;
    LA_CUDA(ctx, cudaMemsetAsync(tickets, 0, (2 + (size_t)groups) * sizeof(int), ctx->stream));
    const long long items = (long long)nb * groups;
    const int cps = ctx->solve_wave > 0 ? ctx->solve_wave : 2;
    const int grid = (int)std::min<long long>(items, (long long)cps * ctx->sm_count);
    solve_wave_kernel<double, EXACT, UPPER, DIVL><<<grid, WT, 0, ctx->stream>>>(
        T, ld, X + c0, ldx, n, nr, nb, groups, tickets, prog, ctx->d_err);
    ctx->launches++;
    LA_TRY(la_check_launch(ctx, "solve_wave_kernel"));
  }
  return LA_OK;
}

template <typename T, bool EXACT>
la_status solve_any(la_ctx ctx, const T* LU, size_t ld, T* X, size_t ldx, int n, int nrhs) {
  if (ctx->solve_wave > 0 && ctx->d_solve_sync && ctx->sm_count > 0 &&
      (nrhs + WC - 1) / WC <= SOLVE_WAVE_MAX_GROUPS)
    return solve_wave<T, EXACT>(ctx, LU, ld, X, ldx, n, nrhs);
  return solve_all<T, EXACT>(ctx, LU, ld, X, ldx, n, nrhs);
}

}  // namespace

// X (>= n rows, pitch ldx) holds B(piv,:) on entry and the solution of the top
// n rows on exit; rows n.. are untouched (the reference's loops stop at n).
la_status launch_lu_solve(la_ctx ctx, bool exact, const double* LU, size_t ld, double* X,
                          size_t ldx, int n, int nrhs) {
  if (n <= 0 || nrhs <= 0) return LA_OK;
  return exact ? solve_any<double, true>(ctx, LU, ld, X, ldx, n, nrhs)
               : solve_any<double, false>(ctx, LU, ld, X, ldx, n, nrhs);
}

// FP32 factors and right-hand sides (the correction solves of iterative refinement).
la_status launch_lu_solve_f32(la_ctx ctx, const float* LU, size_t ld, float* X, size_t ldx, int n,
                              int nrhs) {
  if (n <= 0 || nrhs <= 0) return LA_OK;
  return solve_any<float, false>(ctx, LU, ld, X, ldx, n, nrhs);
}

// One triangle of a solve by the wavefront kernel: lower (unit diagonal, or
// divide = true for a non-unit one) or upper (always divides). The Cholesky
// solves use it (cholesky.rs:123-141).
la_status launch_tri_wave(la_ctx ctx, bool exact, bool upper, bool divide, const double* T,
                          size_t ld, double* X, size_t ldx, int n, int nrhs) {
  if (n <= 0 || nrhs <= 0) return LA_OK;
  if (!ctx->d_solve_sync || ctx->sm_count <= 0) return LA_UNSUPPORTED;
  if (upper)
    return exact ? tri_wave<true, true, false>(ctx, T, ld, X, ldx, n, nrhs)
                 : tri_wave<false, true, false>(ctx, T, ld, X, ldx, n, nrhs);
  if (divide)
    return exact ? tri_wave<true, false, true>(ctx, T, ld, X, ldx, n, nrhs)
                 : tri_wave<false, false, true>(ctx, T, ld, X, ldx, n, nrhs);
  return exact ? tri_wave<true, false, false>(ctx, T, ld, X, ldx, n, nrhs)
               : tri_wave<false, false, false>(ctx, T, ld, X, ldx, n, nrhs);
}
