// Triangular solves of LUDecomposition::solve (src/decomp/lu.rs:256-275),
// blocked by SB = 16 rows, one launch per block step.
//
// Forward (unit L, lu.rs:257-263), step for the finished block [k0, k1):
//   tile 0    : rows of the next block [k1, k2): take the terms of block
//               [k0, k1), then solve the diagonal block (16 sequential steps)
//   tiles 1.. : rows [k2, n): take the terms of block [k0, k1)
// Backward (U, lu.rs:266-275) mirrors it from the bottom, with the division by
// u_kk when a row becomes final.
// The critical path per step is one small tile, while the bulk of the
// update is spread over all SMs. grid.y splits the right-hand sides into
// 32-column chunks.
//
// EXACT applies each term as x_i = x_i - x_k * l_ik without fusion in the
// reference's order (ascending k forward, descending k backward); FAST uses FMA.
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
        if (ty == (k % (ST / CT))) xt[k][tx] = xt[k][tx] / dg[k][k];
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

}  // namespace

// X (>= n rows, pitch ldx) holds B(piv,:) on entry and the solution of the top
// n rows on exit; rows n.. are untouched (the reference's loops stop at n).
la_status launch_lu_solve(la_ctx ctx, bool exact, const double* LU, size_t ld, double* X,
                          size_t ldx, int n, int nrhs) {
  if (n <= 0 || nrhs <= 0) return LA_OK;
  return exact ? solve_all<double, true>(ctx, LU, ld, X, ldx, n, nrhs)
               : solve_all<double, false>(ctx, LU, ld, X, ldx, n, nrhs);
}

// FP32 factors and right-hand sides (the correction solves of iterative refinement).
la_status launch_lu_solve_f32(la_ctx ctx, const float* LU, size_t ld, float* X, size_t ldx, int n,
                              int nrhs) {
  if (n <= 0 || nrhs <= 0) return LA_OK;
  return solve_all<float, false>(ctx, LU, ld, X, ldx, n, nrhs);
}
