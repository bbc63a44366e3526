// FP32 panel factorization on one thread-block cluster (mixed-precision LU).
//
// Same algorithm as lu_panel.cu (partial pivoting with the reference's pivot
// rule, lu.rs:132-160: first row of maximal |v|, NaN rules, scaling by the
// pivot), but the rows of the tall panel live in the shared memory of the
// C CTAs of one cluster (C = 16 where the GPU allows it, else 8), and the
// per-column exchange goes through distributed shared memory:
//   1. each CTA writes its local candidate (key, position, finished row) and,
//      if it owns row j, that row, into its own shared memory (double-buffered
//      by column parity);
//   2. hardware cluster barrier (arrive.release / wait.acquire);
//   3. every CTA reads the C candidates and then the winner's row and row j
//      from the owning CTAs' shared memory (ld.shared::cluster);
//   4. swap, scale and rank-1 update locally.
// One cluster barrier per column and no global-memory round trips; the FP32
// update work per column is small. A last cluster barrier keeps every CTA's
// shared memory alive until all remote reads are done.
#include "la_internal.cuh"

namespace {

constexpr int CW = 32;      // panel width
constexpr int CP = CW + 1;  // padded row pitch in shared memory
constexpr int CT = 256;     // threads per CTA

__device__ __forceinline__ uint32_t cta_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" :::
                   "memory");
}
__device__ __forceinline__ uint32_t remote_addr(const void* local, uint32_t rank) {
  uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(local)), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float ld_remote_f32(uint32_t addr) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ int ld_remote_s32(uint32_t addr) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}

// Integer pivot keys (bits(|v|) + 1; NaN below the diagonal 0, NaN on it the
// maximum): the reference's strict '>' first-maximum rule with integer compares.
__device__ __forceinline__ unsigned ckey(float v, int pos, int j) {
  const unsigned a = __float_as_uint(v) & 0x7fffffffu;
  if (a > 0x7f800000u) return pos == j ? 0xffffffffu : 0u;
  return a + 1u;
}
__device__ __forceinline__ bool cbetter(unsigned ka, int pa, unsigned kb, int pb) {
  if (pb < 0) return pa >= 0;
  if (pa < 0) return false;
  return ka > kb || (ka == kb && pa < pb);
}

struct ClusterPanelArgs {
  float* A;
  size_t ld;
  int m, j0, jb, rpc;
  int* ipiv;
  int* swaps;
};

__global__ void __launch_bounds__(CT, 1) panel_cluster_kernel(ClusterPanelArgs p) {
  extern __shared__ __align__(16) float csm[];
  __shared__ unsigned s_key[2];
  __shared__ int s_pos[2];
  __shared__ float s_crow[2][CW];
  __shared__ float s_drow[2][CW];
  __shared__ float urow[CW];
  __shared__ float drow[CW];
  __shared__ unsigned red_k[CT / 32];
  __shared__ int red_p[CT / 32];
  __shared__ int s_win;
  __shared__ int s_pivs[CW];
  __shared__ float s_scale;

  const int g = (int)cta_rank();
  const int C = (int)(gridDim.x);  // one cluster per launch
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rpc = p.rpc, jb = p.jb;
  float* va = csm;        // [rpc][CP]
  float* lrow = csm + (size_t)rpc * CP;
  const int row0 = p.j0 + g * rpc;
  const int nrows = max(0, min(rpc, p.m - row0));

  for (int idx = tid; idx < rpc * CW; idx += CT) {
    int r = idx / CW, c = idx % CW;
    va[r * CP + c] = (r < nrows && c < jb) ? p.A[(size_t)(row0 + r) * p.ld + p.j0 + c] : 0.f;
  }
  __syncthreads();

  for (int c = 0; c < jb; c++) {
    const int j = p.j0 + c, par = c & 1;
    unsigned bk = 0u;
    int bp = -1;
    for (int r = max(0, j - row0) + tid; r < nrows; r += CT) {
      const int pos = row0 + r;
      const unsigned k = ckey(va[r * CP + c], pos, j);
      if (cbetter(k, pos, bk, bp)) { bk = k; bp = pos; }
    }
    for (int off = 16; off > 0; off >>= 1) {
      unsigned ok = __shfl_down_sync(0xffffffffu, bk, off);
      int op = __shfl_down_sync(0xffffffffu, bp, off);
      if (cbetter(ok, op, bk, bp)) { bk = ok; bp = op; }
    }
    if (lane == 0) { red_k[warp] = bk; red_p[warp] = bp; }
    __syncthreads();
    if (warp == 0) {
      bk = lane < CT / 32 ? red_k[lane] : 0u;
      bp = lane < CT / 32 ? red_p[lane] : -1;
      for (int off = 4; off > 0; off >>= 1) {
        unsigned ok = __shfl_down_sync(0xffffffffu, bk, off);
        int op = __shfl_down_sync(0xffffffffu, bp, off);
        if (cbetter(ok, op, bk, bp)) { bk = ok; bp = op; }
      }
      if (lane == 0) { s_key[par] = bk; s_pos[par] = bp; s_win = bp; }
    }
    __syncthreads();
    if (tid < CW) {
      const int cp = s_win;
      if (cp >= 0) s_crow[par][tid] = va[(cp - row0) * CP + tid];
      if (j >= row0 && j < row0 + nrows) s_drow[par][tid] = va[(j - row0) * CP + tid];
    }
    cluster_sync();

    // Winner over the cluster: lane q reads CTA q's candidate.
    if (warp == 0) {
      unsigned k = 0u;
      int ps = -1;
      if (lane < C) {
        k = (unsigned)ld_remote_s32(remote_addr(&s_key[par], lane));
        ps = ld_remote_s32(remote_addr(&s_pos[par], lane));
      }
      for (int off = 16; off > 0; off >>= 1) {
        unsigned ok = __shfl_down_sync(0xffffffffu, k, off);
        int op = __shfl_down_sync(0xffffffffu, ps, off);
        if (cbetter(ok, op, k, ps)) { k = ok; ps = op; }
      }
      if (lane == 0) {
        s_win = ps;
        s_pivs[c] = ps;
        if (g == 0) p.ipiv[j] = ps;
      }
    }
    __syncthreads();
    const int piv = s_win;
    if (tid < CW) {
      urow[tid] = ld_remote_f32(remote_addr(&s_crow[par][tid], (piv - p.j0) / rpc));
    } else if (tid < 2 * CW) {
      const int t = tid - CW;
      drow[t] = ld_remote_f32(remote_addr(&s_drow[par][t], (j - p.j0) / rpc));
    }
    __syncthreads();
    if (tid == 0) {
      const float d = urow[c];
      s_scale = d != 0.f ? 1.f / d : 1.f;
    }
    if (tid < CW) {
      if (piv != j && piv >= row0 && piv < row0 + nrows) va[(piv - row0) * CP + tid] = drow[tid];
      if (j >= row0 && j < row0 + nrows) va[(j - row0) * CP + tid] = urow[tid];
    }
    __syncthreads();
    const int first = max(0, j + 1 - row0);
    const int cnt = nrows - first;
    const float d = urow[c], sc = s_scale;
    for (int q = tid; q < cnt; q += CT) {
      const int r = first + q;
      const float v = va[r * CP + c];
      const float l = d != 0.f ? v * sc : v;
      va[r * CP + c] = l;
      lrow[r] = l;
    }
    __syncthreads();
    const int cc = c + 1 + (tid & (CW - 1));
    if (cc < jb) {
      const float u = urow[cc];
      for (int q = tid / CW; q < cnt; q += CT / CW) {
        const int r = first + q;
        va[r * CP + cc] = fmaf(-lrow[r], u, va[r * CP + cc]);
      }
    }
    __syncthreads();
  }
  cluster_sync();  // remote reads of the last column are done everywhere

  for (int idx = tid; idx < nrows * CW; idx += CT) {
    int r = idx / CW, c = idx % CW;
    if (c < jb) p.A[(size_t)(row0 + r) * p.ld + p.j0 + c] = va[r * CP + c];
  }
  if (g == 0 && tid == 0) {
    int cnt = 0;
    int* dst = p.swaps + 1;
    int* src = p.swaps + 1 + 2 * MAX_PANEL_W;
    auto find_or_add = [&](int pos) {
      for (int q = 0; q < cnt; q++)
        if (dst[q] == pos) return q;
      dst[cnt] = pos;
      src[cnt] = pos;
      return cnt++;
    };
    for (int c = 0; c < jb; c++) {
      int a = find_or_add(p.j0 + c);
      int b = find_or_add(s_pivs[c]);
      int t = src[a];
      src[a] = src[b];
      src[b] = t;
    }
    int k = 0;
    for (int q = 0; q < cnt; q++)
      if (src[q] != dst[q]) { dst[k] = dst[q]; src[k] = src[q]; k++; }
    p.swaps[0] = k;
  }
}

}  // namespace

// Returns LA_UNSUPPORTED (without launching) when the panel does not fit one
// cluster; the caller then uses the cooperative kernel.
la_status launch_panel_cluster_f32(la_ctx ctx, float* A, size_t ld, int m, int j0, int jb,
                                   int* d_ipiv) {
  const int R = m - j0;
  if (R <= 0 || jb <= 0) return LA_OK;
  if (jb > CW) return LA_UNSUPPORTED;
  static int cluster = -1;  // 16, 8 or 0 (no cluster launch possible)
  static size_t max_smem = 0;
  if (cluster < 0) {
    cluster = 0;
    max_smem = ctx->smem_optin - 2048;  // room for the static buffers
    if (cudaFuncSetAttribute(panel_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed,
                             1) != cudaSuccess ||
        cudaFuncSetAttribute(panel_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)max_smem) != cudaSuccess) {
      cudaGetLastError();
      max_smem = 0;
    }
    for (int c : {16, 8}) {
      if (max_smem == 0) break;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(CT);
      cfg.dynamicSmemBytes = max_smem;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = c;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, panel_cluster_kernel, &cfg) == cudaSuccess &&
          nclusters >= 1) {
        cluster = c;
        break;
      }
      cudaGetLastError();
    }
  }
  if (cluster == 0) return LA_UNSUPPORTED;
  const int rpc = (R + cluster - 1) / cluster;
  const size_t smem = (size_t)rpc * (CP + 1) * sizeof(float);
  if (smem > max_smem) return LA_UNSUPPORTED;

  ClusterPanelArgs a;
  a.A = A;
  a.ld = ld;
  a.m = m;
  a.j0 = j0;
  a.jb = jb;
  a.rpc = rpc;
  a.ipiv = d_ipiv;
  a.swaps = ctx->d_swaps;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster);
  cfg.blockDim = dim3(CT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, panel_cluster_kernel, a);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaLaunchKernelEx(panel_cluster)");
  ctx->launches++;
  return LA_OK;
}
