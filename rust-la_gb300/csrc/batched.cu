// Batched solves of many small, unevenly sized systems (not in the reference;
// each system is LUDecomposition::new + solve, lu.rs:104-278, on its own).
//
// One persistent kernel per precision: every CTA takes the next system from an
// atomic work queue (descriptors sorted by decreasing n^3 on the host, so
// the largest systems start first and the tail is short), then
//   loads A_i (FP64 in HBM) into its working matrix: shared memory when it fits,
//   else the CTA's slice of a global scratch buffer (L2-resident at these sizes);
//   factors it with partial pivoting (the reference's first-maximum pivot rule)
//   by right-looking rank-1 updates over a 16 x 16 thread grid;
//   solves for B_i and writes X_i.
// MIXED factors in FP32 and then refines in FP64 per system: r = b - A x
// with A_i read again in FP64, d = LU32 \ r, x += d, until the normwise
// backward error <= tol or max_iters; systems that do not converge are flagged
// for the FP64 pass, which the same graph runs afterwards over flagged systems
// only. All state is per CTA; no CTA waits on another.
#include "la_internal.cuh"

namespace {

constexpr int BT = 256;  // threads per CTA (16 x 16 update grid)

struct SysDesc {
  long long a;     // offset of A_i (n x n, row-major) in the A buffer, elements
  long long b;     // offset of B_i / X_i (n x nrhs, row-major), elements
  int n, nrhs;
};

template <typename T>
__device__ __forceinline__ unsigned long long bkey(T v, int pos, int j) {
  if (sizeof(T) == 8) {
    const unsigned long long a = (unsigned long long)__double_as_longlong((double)v) &
                                 0x7fffffffffffffffull;
    if (a > 0x7ff0000000000000ull) return pos == j ? ~0ull : 0ull;
    return a + 1ull;
  } else {
    const unsigned a = __float_as_uint((float)v) & 0x7fffffffu;
    if (a > 0x7f800000u) return pos == j ? ~0ull : 0ull;
    return (unsigned long long)a + 1ull;
  }
}

__device__ __forceinline__ bool bbetter(unsigned long long ka, int pa, unsigned long long kb,
                                        int pb) {
  if (pb < 0) return pa >= 0;
  if (pa < 0) return false;
  return ka > kb || (ka == kb && pa < pb);
}

// Blocked right-looking LU with partial pivoting of M (n x n, pitch p), panel
// width pb (<= 16): piv[j] = the row swapped with j at step j.
//   panel  : columns [j0, j1) over rows >= j0, rank-1 updates inside the
//            panel; each pivot swap moves the whole row (lu.rs:140-145)
//   U12    : rows [j0, j1), columns >= j1, one thread per column
//   A22   -= L21 U12 with K = pb: each thread keeps its row's L21 entries in
//            registers and reads U12 from shared memory, so every element of
//            A22 is read and written once per panel (matters when M lives in
//            global scratch).
// stage points at shared memory for L21 / U12 when M is in global memory
// (nullptr: read them from M itself).
template <typename T>
__device__ void block_lu(T* M, int p, int n, int pb, int* piv, unsigned long long* rk, int* rp,
                         int* s_int, T* stage) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tx = tid & 15, ty = tid >> 4;
  for (int j0 = 0; j0 < n; j0 += pb) {
    const int jb = min(pb, n - j0), j1 = j0 + jb;
    // The panel's rows as (R, pitch rp_, column offset co, columns swapped sw):
    // M itself when it is in shared memory, else a staged copy of the panel,
    // so that the pivot steps never wait on L2.
    T* R;
    int rpit, co, sw;
    if (stage) {
      R = stage;  // [rows][17]
      rpit = 17;
      co = 0;
      sw = jb;
      for (int idx = tid; idx < (n - j0) * jb; idx += BT) {
        const int r = idx / jb, c = idx % jb;
        R[r * 17 + c] = M[(j0 + r) * p + j0 + c];
      }
      __syncthreads();
    } else {
      R = M + j0 * p;
      rpit = p;
      co = j0;
      sw = n;
    }
    for (int j = j0; j < j1; j++) {
      const int jr = j - j0, jc = co + j - j0;  // row / column of step j in R
      unsigned long long bk = 0ull;
      int bp = -1;
      for (int r = j + tid; r < n; r += BT) {
        const unsigned long long k = bkey<T>(R[(r - j0) * rpit + jc], r, j);
        if (bbetter(k, r, bk, bp)) { bk = k; bp = r; }
      }
      for (int off = 16; off > 0; off >>= 1) {
        unsigned long long ok = __shfl_down_sync(0xffffffffu, bk, off);
        int op = __shfl_down_sync(0xffffffffu, bp, off);
        if (bbetter(ok, op, bk, bp)) { bk = ok; bp = op; }
      }
      if (lane == 0) { rk[warp] = bk; rp[warp] = bp; }
      __syncthreads();
      if (tid == 0) {
        for (int w = 1; w < BT / 32; w++)
          if (bbetter(rk[w], rp[w], bk, bp)) { bk = rk[w]; bp = rp[w]; }
        s_int[0] = bp;
        piv[j] = bp;
      }
      __syncthreads();
      const int pr = s_int[0] - j0;
      if (pr != jr)
        for (int c = tid; c < sw; c += BT) {
          T t = R[jr * rpit + c];
          R[jr * rpit + c] = R[pr * rpit + c];
          R[pr * rpit + c] = t;
        }
      __syncthreads();
      const T d = R[jr * rpit + jc];
      const T sc = d != T(0) ? T(1) / d : T(1);
      for (int r = jr + 1 + tid; r < n - j0; r += BT) {
        const T v = R[r * rpit + jc];
        R[r * rpit + jc] = d != T(0) ? v * sc : v;
      }
      __syncthreads();
      const int w = j1 - j - 1;  // remaining panel columns
      if (w > 0)
        for (int idx = tid; idx < (n - j - 1) * w; idx += BT) {
          const int r = jr + 1 + idx / w, c = jc + 1 + idx % w;
          R[r * rpit + c] = fma(-R[r * rpit + jc], R[jr * rpit + c], R[r * rpit + c]);
        }
      __syncthreads();
    }
    if (stage) {
      // Panel back to M, and its row swaps (in order) on the other columns.
      for (int idx = tid; idx < (n - j0) * jb; idx += BT) {
        const int r = idx / jb, c = idx % jb;
        M[(j0 + r) * p + j0 + c] = R[r * 17 + c];
      }
      for (int c = tid; c < n; c += BT) {
        if (c >= j0 && c < j1) continue;
        for (int k = j0; k < j1; k++) {
          const int q = piv[k];
          if (q != k) {
            T t = M[k * p + c];
            M[k * p + c] = M[q * p + c];
            M[q * p + c] = t;
          }
        }
      }
      __syncthreads();
    }
    if (j1 >= n) break;
    // U12 = L11^-1 A12: each thread owns whole columns.
    for (int c = j1 + tid; c < n; c += BT)
      for (int k = 0; k < jb; k++) {
        const T u = M[(j0 + k) * p + c];
        for (int i = k + 1; i < jb; i++)
          M[(j0 + i) * p + c] = fma(-M[(j0 + i) * p + j0 + k], u, M[(j0 + i) * p + c]);
      }
    __syncthreads();
    const int nr = n - j1;  // trailing size
    const T* Lb;
    const T* Ub;
    int ldl, ldu;
    if (stage) {
      T* ls = stage;               // [256][16] (reuses the panel staging area)
      T* us = stage + 256 * 17;    // [16][256]
      for (int idx = tid; idx < nr * jb; idx += BT) {
        const int r = idx / jb, k = idx % jb;
        ls[r * 16 + k] = M[(j1 + r) * p + j0 + k];
      }
      for (int idx = tid; idx < jb * nr; idx += BT) {
        const int k = idx / nr, c = idx % nr;
        us[k * 256 + c] = M[(j0 + k) * p + j1 + c];
      }
      __syncthreads();
      Lb = ls; ldl = 16; Ub = us; ldu = 256;
    } else {
      Lb = M + j1 * p + j0; ldl = p; Ub = M + j0 * p + j1; ldu = p;
    }
    for (int r = ty; r < nr; r += 16) {
      T l[16];
#pragma unroll
      for (int k = 0; k < 16; k++) l[k] = k < jb ? Lb[r * ldl + k] : T(0);
      T* mrow = M + (j1 + r) * p + j1;
      for (int c = tx; c < nr; c += 16) {
        T acc = mrow[c];
#pragma unroll
        for (int k = 0; k < 16; k++)
          if (k < jb) acc = fma(-l[k], Ub[k * ldu + c], acc);
        mrow[c] = acc;
      }
    }
    __syncthreads();
  }
}

// X (n x nrhs, pitch px) <- U^-1 L^-1 P X with the factors in M (rows in
// parallel over the CTA, one step per row).
template <typename T, typename TX>
__device__ void block_solve(const T* M, int p, int n, const int* piv, TX* X, int px, int nrhs) {
  const int tid = threadIdx.x;
  // Row swaps in order (the swap list replayed in order is the reference's
  // permutation, lu.rs:245-254).
  if (tid < nrhs)
    for (int j = 0; j < n; j++) {
      const int q = piv[j];
      if (q != j) {
        TX t = X[j * px + tid];
        X[j * px + tid] = X[q * px + tid];
        X[q * px + tid] = t;
      }
    }
  __syncthreads();
  for (int k = 0; k < n; k++) {
    for (int idx = tid; idx < (n - k - 1) * nrhs; idx += BT) {
      const int i = k + 1 + idx / nrhs, c = idx % nrhs;
      X[i * px + c] = fma(-(TX)M[i * p + k], X[k * px + c], X[i * px + c]);
    }
    __syncthreads();
  }
  for (int k = n - 1; k >= 0; k--) {
    if (tid < nrhs) X[k * px + tid] = X[k * px + tid] / (TX)M[k * p + k];
    __syncthreads();
    for (int idx = tid; idx < k * nrhs; idx += BT) {
      const int i = idx / nrhs, c = idx % nrhs;
      X[i * px + c] = fma(-(TX)M[i * p + k], X[k * px + c], X[i * px + c]);
    }
    __syncthreads();
  }
}

struct BatchArgs {
  const double* A;
  const double* B;
  double* X;
  const SysDesc* desc;
  int count;
  int* queue;        // work counter (zeroed before the launch)
  int* status;       // per system (sorted order): iterations, < 0 = not converged
  double* eta;       // per system: final backward error (MIXED) or -1
  void* scratch;     // per-CTA global working matrices for systems that do not fit
  size_t scratch_elems;  // elements per CTA slice
  int smem_n;        // largest n whose working matrix fits in shared memory
  int max_iters;
  double tol;
  int only_flagged;  // FP64 pass: process only systems with status < 0
  int panel;         // panel width of the per-system blocked LU (<= 16)
};

template <typename T, bool MIXED>
__global__ void __launch_bounds__(BT) batched_kernel(BatchArgs a) {
  extern __shared__ __align__(16) double bsm[];
  __shared__ unsigned long long rk[BT / 32];
  __shared__ int rp[BT / 32];
  __shared__ int s_int[2];
  __shared__ T s_t[2];
  __shared__ int s_sys;
  __shared__ double s_norm[1 + 3 * 4];
  __shared__ int s_done;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_sys = atomicAdd(a.queue, 1);
    __syncthreads();
    const int sidx = s_sys;
    if (sidx >= a.count) return;
    if (a.only_flagged && a.status[sidx] >= 0) { __syncthreads(); continue; }
    const SysDesc d = a.desc[sidx];
    const int n = d.n, nrhs = d.nrhs;
    const int p = n + 1;  // padded pitch
    const bool in_smem = n <= a.smem_n;
    T* M = in_smem ? reinterpret_cast<T*>(bsm)
                   : reinterpret_cast<T*>(a.scratch) + (size_t)blockIdx.x * a.scratch_elems;
    // Shared-memory layout after the matrix (sized for n <= 256, nrhs <= 4):
    // piv (256 int), then vectors.
    char* tail = reinterpret_cast<char*>(bsm) + (in_smem ? ((size_t)n * p * sizeof(T) + 15) / 16 * 16 : 0);
    int* piv = reinterpret_cast<int*>(tail);
    double* xv = reinterpret_cast<double*>(tail + 256 * sizeof(int));  // n x 4 FP64 (solution)
    double* rv = xv + 256 * 4;                                          // n x 4 FP64 (residual)
    float* dv = reinterpret_cast<float*>(rv + 256 * 4);                 // n x 4 FP32 (correction)
    const double* Ai = a.A + d.a;
    const double* Bi = a.B + d.b;
    double* Xi = a.X + d.b;

    for (int idx = tid; idx < n * n; idx += BT) M[(idx / n) * p + idx % n] = (T)Ai[idx];
    for (int idx = tid; idx < n * nrhs; idx += BT) xv[idx] = Bi[idx];
    __syncthreads();
    // L21/U12 staging for global-resident matrices: after the vectors.
    T* stage = in_smem ? nullptr : reinterpret_cast<T*>(dv + 256 * 4);
    block_lu<T>(M, p, n, a.panel, piv, rk, rp, s_int, stage);

    if (!MIXED) {
      block_solve<T, double>(M, p, n, piv, xv, nrhs, nrhs);
      for (int idx = tid; idx < n * nrhs; idx += BT) Xi[idx] = xv[idx];
      if (tid == 0) { a.status[sidx] = 0; a.eta[sidx] = -1.0; }
      __syncthreads();
      continue;
    }
    // ---- FP64 refinement with the FP32 factors ----
    // ||A||_inf (row sums, one warp per row), ||b_j||_inf
    if (tid == 0) for (int q = 0; q < 1 + 3 * 4; q++) s_norm[q] = 0.0;
    __syncthreads();
    {
      const int lane = tid & 31, warp = tid >> 5;
      for (int r = warp; r < n; r += BT / 32) {
        double s = 0.0;
        for (int k = lane; k < n; k += 32) s += fabs(Ai[(size_t)r * n + k]);
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (lane == 0)
          atomicMax(reinterpret_cast<unsigned long long*>(&s_norm[0]),
                    (unsigned long long)__double_as_longlong(s));
      }
    }
    for (int idx = tid; idx < n * nrhs; idx += BT) {
      atomicMax(reinterpret_cast<unsigned long long*>(&s_norm[1 + 2 * 4 + idx % nrhs]),
                (unsigned long long)__double_as_longlong(fabs(Bi[idx])));
      rv[idx] = Bi[idx];
      xv[idx] = 0.0;
    }
    __syncthreads();
    int it = 0;
    double eta = INFINITY, prev = INFINITY;
    bool ok = false;
    for (;;) {
      // eta from r (rmax in s_norm[1..4]) and x (xmax in s_norm[5..8])
      if (tid < 8) s_norm[1 + tid] = 0.0;
      __syncthreads();
      for (int idx = tid; idx < n * nrhs; idx += BT) {
        const int c = idx % nrhs;
        atomicMax(reinterpret_cast<unsigned long long*>(&s_norm[1 + c]),
                  (unsigned long long)__double_as_longlong(fabs(rv[idx])));
        atomicMax(reinterpret_cast<unsigned long long*>(&s_norm[1 + 4 + c]),
                  (unsigned long long)__double_as_longlong(fabs(xv[idx])));
      }
      __syncthreads();
      eta = 0.0;
      for (int c = 0; c < nrhs; c++) {
        const double den = s_norm[0] * s_norm[1 + 4 + c] + s_norm[1 + 8 + c];
        const double v = den > 0 ? s_norm[1 + c] / den : (s_norm[1 + c] > 0 ? INFINITY : 0.0);
        if (!(v <= eta)) eta = v;
      }
      if (eta <= a.tol) { ok = true; break; }
      if (it >= a.max_iters || !(eta < 0.9 * prev)) break;
      prev = eta;
      it++;
      // d = LU32 \ (r / rmax), in FP32
      for (int idx = tid; idx < n * nrhs; idx += BT) {
        const double s = s_norm[1 + idx % nrhs];
        dv[idx] = s > 0 ? (float)(rv[idx] / s) : 0.f;
      }
      __syncthreads();
      block_solve<T, float>(M, p, n, piv, dv, nrhs, nrhs);
      for (int idx = tid; idx < n * nrhs; idx += BT) xv[idx] += (double)dv[idx] * s_norm[1 + idx % nrhs];
      __syncthreads();
      // r = b - A x in FP64: one warp per row, lanes along the row (coalesced)
      {
        const int lane = tid & 31, warp = tid >> 5;
        for (int r = warp; r < n; r += BT / 32) {
          const double* ar = Ai + (size_t)r * n;
          double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
          for (int k = lane; k < n; k += 32) {
            const double av = ar[k];
            const double* xk = xv + k * nrhs;
            s0 = fma(av, xk[0], s0);
            if (nrhs > 1) s1 = fma(av, xk[1], s1);
            if (nrhs > 2) s2 = fma(av, xk[2], s2);
            if (nrhs > 3) s3 = fma(av, xk[3], s3);
          }
          for (int off = 16; off > 0; off >>= 1) {
            s0 += __shfl_down_sync(0xffffffffu, s0, off);
            s1 += __shfl_down_sync(0xffffffffu, s1, off);
            s2 += __shfl_down_sync(0xffffffffu, s2, off);
            s3 += __shfl_down_sync(0xffffffffu, s3, off);
          }
          if (lane == 0) {
            rv[r * nrhs] = Bi[(size_t)r * nrhs] - s0;
            if (nrhs > 1) rv[r * nrhs + 1] = Bi[(size_t)r * nrhs + 1] - s1;
            if (nrhs > 2) rv[r * nrhs + 2] = Bi[(size_t)r * nrhs + 2] - s2;
            if (nrhs > 3) rv[r * nrhs + 3] = Bi[(size_t)r * nrhs + 3] - s3;
          }
        }
      }
      __syncthreads();
    }
    for (int idx = tid; idx < n * nrhs; idx += BT) Xi[idx] = xv[idx];
    if (tid == 0) {
      a.status[sidx] = ok ? it : -1 - it;
      a.eta[sidx] = eta;
    }
    __syncthreads();
    (void)s_done;
  }
}

// Upper bound of the kernel's static shared memory (reductions, norms, ids).
constexpr size_t batch_static_smem() { return 1024; }

// Shared memory of the vectors after the matrix: pivots, x, r (FP64), d (FP32).
constexpr size_t tail_bytes() {
  return 256 * sizeof(int) + 2 * 256 * 4 * sizeof(double) + 256 * 4 * sizeof(float);
}

template <typename T, bool MIXED>
size_t smem_for(int n) {
  const size_t mat = ((size_t)n * (n + 1) * sizeof(T) + 15) / 16 * 16;
  return mat + tail_bytes();
}

// Staging for the panel (256 x 17), then L21 / U12 (global-resident matrices)
// after the vectors.
template <typename T>
size_t stage_bytes() {
  return (256 * 17 + 16 * 256) * sizeof(T);
}

}  // namespace

struct la_batch_plan_s {
  la_ctx ctx;
  int count = 0, mode = 0, threads = BT, ctas_per_sm = 1;
  double tol = 1e-14;
  int max_iters = 10;
  const double *A = nullptr, *B = nullptr;
  double* X = nullptr;
  SysDesc* d_desc = nullptr;
  int* d_queue = nullptr;
  int* d_status = nullptr;
  double* d_eta = nullptr;
  void* d_scratch = nullptr;
  int* d_perm = nullptr;  // sorted position -> caller's system index (host copy below)
  std::vector<int> perm;
  size_t smem = 0, scratch_elems = 0;
  int smem_n = 0, grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

template <typename T, bool MIXED>
la_status launch_batch(la_batch_plan_s* pl, int* queue, int only_flagged, size_t smem, int smem_n,
                       void* scratch, size_t scratch_elems) {
  la_ctx ctx = pl->ctx;
  BatchArgs a;
  a.A = pl->A;
  a.B = pl->B;
  a.X = pl->X;
  a.desc = pl->d_desc;
  a.count = pl->count;
  a.queue = queue;
  a.status = pl->d_status;
  a.eta = pl->d_eta;
  a.scratch = scratch;
  a.scratch_elems = scratch_elems;
  a.smem_n = smem_n;
  a.max_iters = pl->max_iters;
  a.tol = pl->tol;
  a.only_flagged = only_flagged;
  a.panel = 16;
  static bool configured = false;  // outside any stream capture (first plan run)
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(batched_kernel<T, MIXED>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(ctx->smem_optin - batch_static_smem()));
    if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaFuncSetAttribute(batched)");
    configured = true;
  }
  batched_kernel<T, MIXED><<<pl->grid, BT, smem, ctx->stream>>>(a);
  ctx->launches++;
  return la_check_launch(ctx, "batched_kernel");
}

// Largest n whose working matrix and vectors fit `budget` bytes of shared memory.
template <typename T, bool MIXED>
int fit_n(size_t budget) {
  int n = 0;
  for (int t = 1; t <= 256; t++)
    if (smem_for<T, MIXED>(t) <= budget) n = t;
  return n;
}

// The whole pipeline (both passes) on the context's stream.
la_status enqueue_plan(la_batch_plan_s* pl) {
  la_ctx ctx = pl->ctx;
  LA_CUDA(ctx, cudaMemsetAsync(pl->d_queue, 0, 2 * sizeof(int), ctx->stream));
  // The per-CTA budget keeps ctas_per_sm CTAs resident per SM.
  if (pl->mode == LA_BATCH_FP64) {
    LA_TRY((launch_batch<double, false>(pl, pl->d_queue, 0, pl->smem, pl->smem_n, pl->d_scratch,
                                        pl->scratch_elems)));
  } else {
    LA_TRY((launch_batch<float, true>(pl, pl->d_queue, 0, pl->smem, pl->smem_n, pl->d_scratch,
                                      pl->scratch_elems)));
    // FP64 pass over systems whose refinement did not converge.
    const size_t budget = pl->smem;
    LA_TRY((launch_batch<double, false>(pl, pl->d_queue + 1, 1, budget,
                                        fit_n<double, false>(budget), pl->d_scratch,
                                        pl->scratch_elems)));
  }
  return LA_OK;
}

}  // namespace

extern "C" {

la_status la_batch_plan_create(la_ctx ctx, const double* d_a, const double* d_b, double* d_x,
                               const la_batch_system* systems, int count, int mode,
                               int ctas_per_sm, double tol, int max_iters, la_batch_plan* out) {
  if (!ctx || !d_a || !d_b || !d_x || !systems || !out || count <= 0) return LA_INVALID;
  if (mode != LA_BATCH_FP64 && mode != LA_BATCH_MIXED) return LA_INVALID;
  if (ctas_per_sm < 1 || ctas_per_sm > 4) return LA_INVALID;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  for (int i = 0; i < count; i++)
    if (systems[i].n < 1 || systems[i].n > 256 || systems[i].nrhs < 1 || systems[i].nrhs > 4)
      return LA_UNSUPPORTED;
  la_batch_plan_s* pl = new (std::nothrow) la_batch_plan_s();
  if (!pl) return LA_NOMEM;
  pl->ctx = ctx;
  pl->count = count;
  pl->mode = mode;
  pl->ctas_per_sm = ctas_per_sm;
  pl->tol = tol;
  pl->max_iters = max_iters;
  pl->A = d_a;
  pl->B = d_b;
  pl->X = d_x;
  // Work queue order: decreasing n (cost ~ n^3), ties by index.
  pl->perm.resize(count);
  for (int i = 0; i < count; i++) pl->perm[i] = i;
  std::stable_sort(pl->perm.begin(), pl->perm.end(),
                   [&](int x, int y) { return systems[x].n > systems[y].n; });
  std::vector<SysDesc> h(count);
  for (int i = 0; i < count; i++) {
    const la_batch_system& s = systems[pl->perm[i]];
    h[i].a = (long long)s.a_offset;
    h[i].b = (long long)s.b_offset;
    h[i].n = s.n;
    h[i].nrhs = s.nrhs;
  }
  // Shared memory per CTA for the requested residency.
  // Per CTA: the opt-in limit less the static part, or the SM's 228 KB shared
  // among ctas_per_sm CTAs (1 KB reserved per CTA).
  const size_t per_cta = (size_t)ctx->smem_optin - batch_static_smem();
  size_t budget = std::min(per_cta, (size_t)(228 * 1024) / ctas_per_sm - 1024 - batch_static_smem());
  // A CTA also needs room for the L21 / U12 staging when a system works in
  // global scratch.
  const size_t need = tail_bytes() + (mode == LA_BATCH_FP64 ? stage_bytes<double>()
                                                             : stage_bytes<double>());
  if (budget < need) {
    delete pl;
    return LA_UNSUPPORTED;
  }
  pl->smem = budget;
  pl->smem_n = mode == LA_BATCH_FP64 ? fit_n<double, false>(budget) : fit_n<float, true>(budget);
  pl->grid = ctx->sm_count * ctas_per_sm;
  pl->scratch_elems = (size_t)256 * 257;
  la_status s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_desc), count * sizeof(SysDesc));
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_queue), 64);
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_status), count * sizeof(int));
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_eta), count * sizeof(double));
  if (s == LA_OK)
    s = la_device_alloc(ctx, &pl->d_scratch, (size_t)pl->grid * pl->scratch_elems * sizeof(double));
  if (s == LA_OK) {
    cudaError_t e = cudaMemcpyAsync(pl->d_desc, h.data(), count * sizeof(SysDesc),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(pl->d_status, 0, count * sizeof(int), ctx->stream);
    if (e != cudaSuccess) s = la_cuda_fail(ctx, e, "batch plan upload");
  }
  if (s == LA_OK) s = la_sync_and_check(ctx, "batch plan");
  // Capture the pipeline in a CUDA graph (attributes are set by a first
  // uncaptured run so capture only records launches).
  if (s == LA_OK) s = enqueue_plan(pl);
  if (s == LA_OK) s = la_sync_and_check(ctx, "batch warm run");
  if (s == LA_OK) {
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    cudaStream_t saved = ctx->stream;
    if (e == cudaSuccess) {
      ctx->stream = cs;
      e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        la_status es = enqueue_plan(pl);
        cudaError_t e2 = cudaStreamEndCapture(cs, &pl->graph);
        if (es != LA_OK) s = es;
        else if (e2 != cudaSuccess) e = e2;
      }
      ctx->stream = saved;
      cudaStreamDestroy(cs);
    }
    if (s == LA_OK && e == cudaSuccess) e = cudaGraphInstantiate(&pl->exec, pl->graph, 0);
    if (s == LA_OK && e != cudaSuccess) s = la_cuda_fail(ctx, e, "batch graph");
  }
  if (s != LA_OK) {
    la_batch_plan_destroy(pl);
    return s;
  }
  *out = pl;
  return LA_OK;
}

la_status la_batch_plan_run(la_batch_plan pl) {
  if (!pl) return LA_INVALID;
  la_ctx ctx = pl->ctx;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  LA_CUDA(ctx, cudaGraphLaunch(pl->exec, ctx->stream));
  return LA_OK;
}

la_status la_batch_plan_stats(la_batch_plan pl, int* iterations, double* eta, int* fell_back) {
  if (!pl) return LA_INVALID;
  la_ctx ctx = pl->ctx;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  std::vector<int> st(pl->count);
  std::vector<double> et(pl->count);
  LA_CUDA(ctx, cudaMemcpyAsync(st.data(), pl->d_status, pl->count * sizeof(int),
                               cudaMemcpyDeviceToHost, ctx->stream));
  LA_CUDA(ctx, cudaMemcpyAsync(et.data(), pl->d_eta, pl->count * sizeof(double),
                               cudaMemcpyDeviceToHost, ctx->stream));
  LA_TRY(la_sync_and_check(ctx, "batch stats"));
  for (int i = 0; i < pl->count; i++) {
    const int orig = pl->perm[i];
    // FP64 pass results carry status 0 and eta -1; refinement keeps its count.
    if (iterations) iterations[orig] = st[i] >= 0 ? st[i] : -1 - st[i];
    if (eta) eta[orig] = et[i];
    if (fell_back) fell_back[orig] = (pl->mode == LA_BATCH_MIXED && et[i] < 0.0) ? 1 : 0;
  }
  return LA_OK;
}

void la_batch_plan_destroy(la_batch_plan pl) {
  if (!pl) return;
  la_ctx ctx = pl->ctx;
  cudaSetDevice(ctx->device);
  if (pl->exec) cudaGraphExecDestroy(pl->exec);
  if (pl->graph) cudaGraphDestroy(pl->graph);
  la_device_free(ctx, pl->d_desc);
  la_device_free(ctx, pl->d_queue);
  la_device_free(ctx, pl->d_status);
  la_device_free(ctx, pl->d_eta);
  la_device_free(ctx, pl->d_scratch);
  cudaStreamSynchronize(ctx->stream);
  delete pl;
}

}  // extern "C"

extern "C" la_status la_batch_autotune(la_ctx ctx, const double* d_a, const double* d_b,
                                       double* d_x, const la_batch_system* systems, int count,
                                       int mode, double tol, int max_iters,
                                       const char* table_path, int* best_ctas_per_sm,
                                       double* best_ms) {
  if (!ctx || !best_ctas_per_sm) return LA_INVALID;
  double mean_n = 0;
  for (int i = 0; i < count; i++) mean_n += systems[i].n;
  mean_n /= std::max(count, 1);
  int best = 1;
  double best_t = INFINITY;
  std::vector<std::pair<int, double>> rows;
  for (int c = 1; c <= 4; c++) {
    la_batch_plan pl = nullptr;
    la_status s = la_batch_plan_create(ctx, d_a, d_b, d_x, systems, count, mode, c, tol,
                                       max_iters, &pl);
    if (s != LA_OK) continue;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double t = INFINITY;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0, ctx->stream);
      la_batch_plan_run(pl);
      cudaEventRecord(e1, ctx->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) break;
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      t = std::min(t, (double)ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    la_batch_plan_destroy(pl);
    rows.push_back({c, t});
    if (t < best_t) { best_t = t; best = c; }
  }
  if (rows.empty()) return LA_CUDA_ERROR;
  if (table_path) {
    FILE* f = fopen(table_path, "a");
    if (f) {
      for (auto& r : rows)
        fprintf(f, "%s %d %.1f %d %.4f\n", mode == LA_BATCH_FP64 ? "fp64" : "mixed", count,
                mean_n, r.first, r.second);
      fclose(f);
    }
  }
  *best_ctas_per_sm = best;
  if (best_ms) *best_ms = best_t;
  return la_sync_and_check(ctx, "batch autotune");
}
