// Panel factorization of the blocked LU: columns [j0, j0+jb) over rows
// [j0, m), with partial pivoting (src/decomp/lu.rs:116-161 restricted to the
// panel's columns).
//
// The tall panel is spread over G co-resident CTAs (cooperative launch); each
// CTA keeps its contiguous chunk of rows in shared memory for the whole panel,
// so the only global traffic per column is one candidate row per CTA. Per
// column j there is exactly one grid barrier:
//   1. each CTA finds its local pivot candidate, first row of max |v| (the
//      reference's strict '>' scan, lu.rs:132-137), and publishes the value,
//      its row position and the full finished row; the owner of row j also
//      publishes row j (it moves to the pivot's place, lu.rs:140-145);
//   2. barrier;
//   3. every CTA picks the same winner (max |v|, then lowest position), takes
//      the pivot row as U's row j, swaps in place, scales its rows below j by
//      the pivot (true division, skipped for a zero pivot, lu.rs:156-160) and
//      applies the rank-1 update to the rest of the panel.
// Candidate buffers are double-buffered by column parity, so a CTA that runs
// ahead never overwrites data a slower CTA is still reading.
//
// EXACT keeps, per element, the original value a and the running sum s of
// l_ik*u_kj (added in ascending k without fusion, lu.rs:124-126) and forms
// v = a - s only when the column is reached (lu.rs:128); finished entries
// carry s = 0 so v = a - 0 = a for them. FAST updates v in place with FMA.
//
// Every wait is bounded: a CTA that waits past the limit (2 s, or the
// context's LA_OPT_WAIT_LIMIT_US) or sees another CTA give up records
// DERR_PANEL_TIMEOUT and returns; the host reports LA_TIMEOUT. A panel launched
// after an error has been recorded returns at once, and so do the kernels that
// would apply its row interchanges (lu_aux.cu).
#include "la_internal.cuh"
#include "swap_compose.cuh"

namespace {

constexpr int PT = 256;  // threads per panel CTA
constexpr unsigned long long WAIT_LIMIT_NS = 2000000000ull;  // 2 s (default)

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_volatile_i32(const int* p) {
  int v;
  asm volatile("ld.volatile.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Grid barrier on a monotonically increasing counter (the pattern of a
// cooperative-groups grid sync: CTA barrier, one thread fences, arrives with a
// release add and polls with acquire loads). Returns false when the wait gave up
// (this CTA timed out or another CTA reported an error).
__device__ bool grid_barrier(unsigned* counter, unsigned target, int* err,
                             unsigned long long wait_ns) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(counter), "r"(1u) : "memory");
    int good = 1;
    unsigned long long t0 = 0;
    unsigned spins = 0;
    while (ld_acquire_u32(counter) < target) {
      if ((++spins & 63u) == 0) {
        if (ld_volatile_i32(err) != 0) { good = 0; break; }
        unsigned long long now = globaltimer_ns();
        if (t0 == 0) t0 = now;
        else if (now - t0 > wait_ns) {
          atomicCAS(err, 0, (int)DERR_PANEL_TIMEOUT);
          good = 0;
          break;
        }
      }
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Ordering key of a pivot candidate, as an integer so that no FP64
// instruction is spent on comparisons (the FP64 pipe is slow on this GPU):
// bits(|v|) + 1 orders like |v| for every non-NaN value. NaN never wins a strict
// '>' test, so a NaN below the diagonal gets 0 (below everything); a NaN on the
// diagonal row j is never displaced, so it gets the maximum (ties go to the
// lowest position, which is j).
__device__ __forceinline__ unsigned long long pivot_key(double v, int pos, int j) {
  const unsigned long long a = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
  if (a > 0x7ff0000000000000ull) return pos == j ? ~0ull : 0ull;
  return a + 1ull;
}
__device__ __forceinline__ unsigned long long pivot_key(float v, int pos, int j) {
  const unsigned a = __float_as_uint(v) & 0x7fffffffu;
  if (a > 0x7f800000u) return pos == j ? ~0ull : 0ull;
  return (unsigned long long)a + 1ull;
}
__device__ __forceinline__ bool better(unsigned long long ka, int pa, unsigned long long kb, int pb) {
  // a beats b: larger key, or equal key and lower position; pb < 0 means empty.
  if (pb < 0) return pa >= 0;
  if (pa < 0) return false;
  return ka > kb || (ka == kb && pa < pb);
}

struct PanelParams {
  void* A;        // element type of the kernel instantiation
  void* S;
  size_t ld;
  int m, j0, jb, rpc, G;
  int* ipiv;
  unsigned* bar;
  unsigned bar_base;  // counter value at kernel start (the counter only grows)
  unsigned stall;     // arrivals added to every barrier target (failure injection; 0)
  unsigned long long wait_ns;  // limit of each barrier wait
  int* err;
  unsigned long long* cand_key;
  int* cand_pos;
  double* cand_row;
  double* diag_a;
  double* diag_s;
  int* swaps;  // [0] = count, then (dest, src) pairs of the composed row moves
  int cstride; // candidate slots per parity (>= G)
};

// T is the element type of the panel (double, or float for the mixed-precision
// LU); the exchange buffers in global memory always hold doubles (exact for
// both). EXACT exists for double only.
template <typename T, bool EXACT>
__global__ void __launch_bounds__(PT) panel_kernel(PanelParams p) {
  extern __shared__ __align__(16) double sm_raw[];
  T* sm = reinterpret_cast<T*>(sm_raw);
  constexpr int W = MAX_PANEL_W;
  const int rpc = p.rpc;
  T* va = sm;                                // [rpc][W]  value (FAST) / a (EXACT)
  T* vs = EXACT ? sm + rpc * W : nullptr;    // [rpc][W]  running sum s (EXACT)
  T* urow = sm + (EXACT ? 2 : 1) * rpc * W;  // [W] pivot row
  T* drow_a = urow + W;                      // [W] row j as published (raw)
  T* drow_s = drow_a + W;                    // [W] its running sums (EXACT)
  T* lrow = drow_s + W;                      // [rpc] multipliers of this step
  __shared__ unsigned long long red_k[PT / 32];
  __shared__ int red_p[PT / 32];
  __shared__ int s_win_pos;
  __shared__ T s_scale;
  __shared__ int s_pivs[W];
  __shared__ int s_atp[SWAP_SLOTS], s_atr[SWAP_SLOTS];
  __shared__ int s_abort;

  const int g = blockIdx.x;
  const int tid = threadIdx.x;
  // An error recorded earlier in this factorization (a wait that gave up):
  // the panel's inputs are not valid, return before touching anything.
  if (tid == 0) s_abort = ld_volatile_i32(p.err);
  __syncthreads();
  if (s_abort) return;
  const int lane = tid & 31, warp = tid >> 5;
  const int jb = p.jb;
  const int row0 = p.j0 + g * rpc;                  // position of local row 0
  const int nrows = max(0, min(rpc, p.m - row0));   // rows owned by this CTA

  for (int idx = tid; idx < rpc * W; idx += PT) {
    int r = idx / W, c = idx % W;
    T a = T(0), s = T(0);
    if (r < nrows && c < jb) {
      size_t off = (size_t)(row0 + r) * p.ld + p.j0 + c;
      a = static_cast<const T*>(p.A)[off];
      if (EXACT) s = static_cast<const T*>(p.S)[off];
    }
    va[idx] = a;
    if (EXACT) vs[idx] = s;
  }
  __syncthreads();

  for (int c = 0; c < jb; c++) {
    const int j = p.j0 + c;
    const int par = c & 1;
    // 1. local candidate over owned rows at positions >= j.
    unsigned long long bk = 0ull;
    int bp = -1;
    for (int r = max(0, j - row0) + tid; r < nrows; r += PT) {
      const int pos = row0 + r;
      const unsigned long long k =
          EXACT ? pivot_key((double)__dsub_rn(va[r * W + c], vs[r * W + c]), pos, j)
                : pivot_key(va[r * W + c], pos, j);
      if (better(k, pos, bk, bp)) { bk = k; bp = pos; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      unsigned long long ok = __shfl_down_sync(0xffffffffu, bk, off);
      int op = __shfl_down_sync(0xffffffffu, bp, off);
      if (better(ok, op, bk, bp)) { bk = ok; bp = op; }
    }
    if (lane == 0) { red_k[warp] = bk; red_p[warp] = bp; }
    __syncthreads();
    if (warp == 0) {
      bk = lane < PT / 32 ? red_k[lane] : 0ull;
      bp = lane < PT / 32 ? red_p[lane] : -1;
#pragma unroll
      for (int off = 4; off > 0; off >>= 1) {
        unsigned long long ok = __shfl_down_sync(0xffffffffu, bk, off);
        int op = __shfl_down_sync(0xffffffffu, bp, off);
        if (better(ok, op, bk, bp)) { bk = ok; bp = op; }
      }
      if (lane == 0) {
        p.cand_key[par * p.cstride + g] = bk;
        p.cand_pos[par * p.cstride + g] = bp;
        s_win_pos = bp;
      }
    }
    __syncthreads();
    // 2. publish the candidate row (finished values) and, if owned, row j.
    {
      const int cp = s_win_pos;
      if (cp >= 0 && tid < W) {
        int r = cp - row0;
        double v = EXACT ? __dsub_rn(va[r * W + tid], vs[r * W + tid]) : (double)va[r * W + tid];
        p.cand_row[((size_t)par * p.cstride + g) * W + tid] = v;
      }
      if (j >= row0 && j < row0 + nrows && tid >= PT - W) {
        const int t = tid - (PT - W);
        const int r = j - row0;
        p.diag_a[par * W + t] = (double)va[r * W + t];
        if (EXACT) p.diag_s[par * W + t] = (double)vs[r * W + t];
      }
    }
    if (!grid_barrier(p.bar, p.bar_base + (unsigned)(p.G * (c + 1)) + p.stall, p.err, p.wait_ns))
      return;

    // 3. global winner (identical in every CTA): one candidate per thread; the
    //    last W threads fetch row j at the same time (needed if it moves here).
    {
      unsigned long long k = 0ull;
      int ps = -1;
      if (tid < p.G) {
        k = __ldcg(p.cand_key + par * p.cstride + tid);
        ps = __ldcg(p.cand_pos + par * p.cstride + tid);
      }
      if (tid >= PT - W) {
        const int t = tid - (PT - W);
        drow_a[t] = (T)__ldcg(p.diag_a + par * W + t);
        if (EXACT) drow_s[t] = (T)__ldcg(p.diag_s + par * W + t);
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        unsigned long long ok = __shfl_down_sync(0xffffffffu, k, off);
        int op = __shfl_down_sync(0xffffffffu, ps, off);
        if (better(ok, op, k, ps)) { k = ok; ps = op; }
      }
      if (lane == 0) { red_k[warp] = k; red_p[warp] = ps; }
      __syncthreads();
      if (warp == 0) {
        k = lane < PT / 32 ? red_k[lane] : 0ull;
        ps = lane < PT / 32 ? red_p[lane] : -1;
#pragma unroll
        for (int off = 4; off > 0; off >>= 1) {
          unsigned long long ok = __shfl_down_sync(0xffffffffu, k, off);
          int op = __shfl_down_sync(0xffffffffu, ps, off);
          if (better(ok, op, k, ps)) { k = ok; ps = op; }
        }
        if (lane == 0) {
          s_win_pos = ps;
          s_pivs[c] = ps;
          if (g == 0) p.ipiv[j] = ps;
        }
      }
      __syncthreads();
    }
    const int piv = s_win_pos;
    const int wg = (piv - p.j0) / rpc;  // CTA that owns the winning row
    if (tid < W) urow[tid] = (T)__ldcg(p.cand_row + ((size_t)par * p.cstride + wg) * W + tid);
    __syncthreads();
    if (tid == 0) {
      const T d = urow[c];
      // FAST scales by the reciprocal (as LAPACK's getf2 does); EXACT divides.
      s_scale = (d != T(0)) ? T(1) / d : T(1);
    }
    // Swap: row j <- pivot row (finished), row piv <- old row j (raw storage).
    if (tid < W) {
      if (piv != j && piv >= row0 && piv < row0 + nrows) {
        const int r = piv - row0;
        va[r * W + tid] = drow_a[tid];
        if (EXACT) vs[r * W + tid] = drow_s[tid];
      }
      if (j >= row0 && j < row0 + nrows) {
        const int r = j - row0;
        va[r * W + tid] = urow[tid];
        if (EXACT) vs[r * W + tid] = T(0);
      }
    }
    __syncthreads();
    // 4a. multipliers l_i = v_i / u_jj for owned rows below j; rows are spread
    //     over all warps (row = lane * 8 + warp) so every SM sub-partition works.
    const int first = max(0, j + 1 - row0);
    const int cnt = nrows - first;
    {
      const T d = urow[c];
      const T sc = s_scale;
      for (int q = lane * (PT / 32) + warp; q < cnt; q += PT) {
        const int r = first + q;
        T v = EXACT ? (T)__dsub_rn(va[r * W + c], vs[r * W + c]) : va[r * W + c];
        T l = (d != T(0)) ? (EXACT ? v / d : v * sc) : v;
        va[r * W + c] = l;
        if (EXACT) vs[r * W + c] = T(0);
        lrow[r] = l;
      }
    }
    __syncthreads();
    // 4b. rank-1 update of the remaining panel columns: thread = (column lane,
    //     row group of 4).
    const int cc = c + 1 + (tid & (W - 1));
    if (cc < jb) {
      const T u = urow[cc];
      for (int q = tid / W; q < cnt; q += PT / W) {
        const int r = first + q;
        const T l = lrow[r];
        if (EXACT)
          vs[r * W + cc] = __dadd_rn(vs[r * W + cc], __dmul_rn(l, u));
        else
          va[r * W + cc] = fma(-l, u, va[r * W + cc]);
      }
    }
    __syncthreads();
  }

  for (int idx = tid; idx < nrows * W; idx += PT) {
    int r = idx / W, c = idx % W;
    if (c < jb) {
      T v = EXACT ? (T)__dsub_rn(va[idx], vs[idx]) : va[idx];
      static_cast<T*>(p.A)[(size_t)(row0 + r) * p.ld + p.j0 + c] = v;
    }
  }
  // Compose this panel's swaps into a list of row moves (dest <- src) for the
  // columns outside the panel (applied by the row-swap kernel).
  if (g == 0 && warp == 0)
    compose_swaps_warp(s_pivs, jb, p.j0, false, nullptr, p.swaps, s_atp, s_atr, lane);
}

}  // namespace

template <typename T>
la_status launch_panel_t(la_ctx ctx, cudaStream_t stream, bool exact, T* A, T* S, size_t ld,
                         int m, int j0, int jb, int* d_ipiv, unsigned* bar_base) {
  const int R = m - j0;
  if (R <= 0 || jb <= 0) return LA_OK;
  if (exact && sizeof(T) != sizeof(double)) return LA_INVALID;
  const int W = MAX_PANEL_W;
  int maxG = ctx->panel_ctas > 0 ? std::min(ctx->panel_ctas, ctx->sm_count) : ctx->sm_count;
  maxG = std::min(maxG, PT);  // one candidate per thread when picking the winner
  maxG = std::min(maxG, ctx->cand_stride);
  // At least 32 rows per CTA: fewer CTAs keep the per-column barrier cheap.
  int G = std::max(1, std::min(maxG, (R + 31) / 32));
  int rpc = (R + G - 1) / G;
  const size_t per_row = (size_t)W * sizeof(T) * (exact ? 2 : 1) + sizeof(T);
  const size_t fixed = (size_t)3 * W * sizeof(T) + 16;
  size_t smem = fixed + per_row * rpc;
  if (smem > ctx->smem_optin) return LA_UNSUPPORTED;
  G = (R + rpc - 1) / rpc;

  PanelParams p;
  p.A = A;
  p.S = S;
  p.ld = ld;
  p.m = m;
  p.j0 = j0;
  p.jb = jb;
  p.rpc = rpc;
  p.G = G;
  p.ipiv = d_ipiv;
  p.bar = ctx->d_bar;
  p.bar_base = *bar_base;
  p.stall = 0;
  if (ctx->inject_panel_stall > 0 && --ctx->inject_panel_stall == 0) p.stall = 1;
  p.wait_ns = ctx->wait_limit_us > 0 ? (unsigned long long)ctx->wait_limit_us * 1000ull
                                     : WAIT_LIMIT_NS;
  p.err = ctx->d_err;
  p.cand_key = reinterpret_cast<unsigned long long*>(ctx->d_cand_abs);
  p.cand_pos = ctx->d_cand_pos;
  p.cand_row = ctx->d_cand_row;
  p.diag_a = ctx->d_diag_a;
  p.diag_s = ctx->d_diag_s;
  p.swaps = ctx->d_swaps;
  p.cstride = ctx->cand_stride;

  void* args[] = {&p};
  const void* fn;
  if (sizeof(T) == sizeof(double))
    fn = exact ? (const void*)panel_kernel<double, true> : (const void*)panel_kernel<double, false>;
  else
    fn = (const void*)panel_kernel<float, false>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaFuncSetAttribute(panel)");
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, PT, smem);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "occupancy(panel)");
  if (per_sm * ctx->sm_count < G) return LA_UNSUPPORTED;
  e = cudaLaunchCooperativeKernel(fn, dim3(G), dim3(PT), args, smem, stream);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaLaunchCooperativeKernel(panel)");
  ctx->launches++;
  *bar_base += (unsigned)(G * jb);
  return la_check_launch(ctx, "panel_kernel");
}

la_status launch_panel(la_ctx ctx, cudaStream_t stream, bool exact, double* A, double* S,
                       size_t ld, int m, int j0, int jb, int* d_ipiv, unsigned* bar_base) {
  return launch_panel_t<double>(ctx, stream, exact, A, S, ld, m, j0, jb, d_ipiv, bar_base);
}

la_status launch_panel_f32(la_ctx ctx, cudaStream_t stream, float* A, size_t ld, int m, int j0,
                           int jb, int* d_ipiv, unsigned* bar_base) {
  return launch_panel_t<float>(ctx, stream, false, A, nullptr, ld, m, j0, jb, d_ipiv, bar_base);
}
