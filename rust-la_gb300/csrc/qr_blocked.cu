// Blocked Householder QR for FAST arithmetic: QRDecomposition::new, get_q and
// solve (src/decomp/qr.rs:26-238) in compact WY form.
//
// The reference's reflection by column k is H_k = I - tau_k v_k v_k', v_k the
// Householder vector it stores (x - a e_k: the diagonal entry u0 = q - a, the
// entries below unchanged). The reflections of a block of QB columns multiply
// to I - V T V' with T upper triangular, and
//   T^-1 = diag(1/tau) + strictly_upper(G),  G = V'V
// (invert the recurrence T_k = [[T, -tau_k T V' v_k], [0, tau_k]] column by
// column). The products T' W and T W are therefore substitutions with G:
//   forward  W2_i = tau_i (W_i - sum_{k<i} G_ki W2_k)   (T' W)
//   backward W2_i = tau_i (W_i - sum_{k>i} G_ik W2_k)   (T W)
// which hold for tau_i = 0 too (a skipped reflection: row and column i of T
// are zero). tau per caller:
//   factorization (qr.rs:60-103): -1/(a u0), 0 where a == 0;
//   get_q (qr.rs:163-189): -1/(rdiag u0), 0 where u0 == 0; blocks in reverse,
//       Q[j:, j:] -= V (T (V' Q[j:, j:]));
//   solve (qr.rs:211-223): 1/u0 (the reference's factor -(dot / u0)); blocks
//       in order, X[j:] -= V (T' (V' X[j:])).
//
// One block of the factorization (columns [j, j + nb), rows [j, m)):
//   qr_panel_kernel    the block's reflections one after another on one
//                      cluster of 16 (or 8) CTAs that hold the rows in shared
//                      memory. One cluster barrier per column: every CTA
//                      publishes to every CTA its partial sums x.x and x.t_c
//                      (the column before its reflection against each later
//                      column of the block) and the owner of the diagonal row
//                      publishes that row; every CTA then sums the parts in
//                      rank order and forms a, u0 = q - a and
//                      u.t_c = x.t_c - a t_c[diag] identically. At the end the
//                      block goes back to A with zeros above the diagonal of
//                      its top square (whose final content is kept in rsave),
//                      V' to its own buffer, a to rdiag and tau.
//   W = V' A[j:, j:]   split-K FP64 GEMM (gemm_f64) and a reduction of the
//                      partial products; W's first nb columns are G.
//   W2 = T' W          qr_tsolve_kernel (one warp per column).
//   A[j:, j+nb:] -= V W2, then the top square restored from rsave.
// G of every block is kept for get_q and solve.
//
// The blocked and the column-by-column FAST forms perform the same reflections
// with differently ordered sums; EXACT arithmetic stays column by column.
#include <algorithm>

#include "la_internal.cuh"

namespace {

constexpr int QB = QR_BLOCK;      // block width
constexpr int QPT = 256;          // panel threads
constexpr int QNBP = QB + 1;      // shared row pitch (odd: column reads without bank conflicts)
constexpr int QMAXCL = 16;        // largest cluster
constexpr int QTS_W = 8;          // warps (columns) per substitution CTA

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
__device__ __forceinline__ void st_remote_f64(uint32_t addr, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}

struct QrPanelArgs {
  double* A;
  size_t ld;
  int m, j, nb, rpc;  // rows [j, m), columns [j, j + nb), rpc rows per CTA
  double* rdiag;
  double* tau;        // [nb]
  double* vt;         // V' (nb x rows, pitch ldv)
  size_t ldv;
  double* rsave;      // the top square's final content (nb x QB)
};

__global__ void __launch_bounds__(QPT, 1) qr_panel_kernel(QrPanelArgs p) {
  extern __shared__ __align__(16) double P[];  // [rpc][QNBP]
  __shared__ double xch[2][QMAXCL][QB];        // partial sums, one slot per source CTA
  __shared__ double own[2][QB];                // the diagonal row: q, then t_c
  __shared__ double red[QPT];
  __shared__ double mine[QB], tot[QB], fac[QB];
  const int tid = threadIdx.x;
  const uint32_t rank = cta_rank();
  const int CL = (int)gridDim.x;  // one cluster per launch
  const int nb = p.nb;
  const int r0 = p.j + (int)rank * p.rpc;      // first global row of this CTA
  const int nr = max(0, min(p.rpc, p.m - r0));  // rows held

  for (int idx = tid; idx < nr * nb; idx += QPT) {
    const int lr = idx / nb, c = idx % nb;
    P[lr * QNBP + c] = p.A[(size_t)(r0 + lr) * p.ld + p.j + c];
  }
  __syncthreads();

  for (int k = 0; k < nb; k++) {
    const int par = k & 1, jc = p.j + k, w = nb - k;
    const int lr0 = max(0, jc - r0);  // first local row at or below the diagonal
    // x (column k) against columns k..nb-1 (the first is x.x). Thread t takes
    // column k + t % w of the rows lr0 + t / w + G i: every lane of an FP64
    // instruction does useful work whatever w is.
    {
      const int G = QPT / w;
      double sacc = 0.0;
      if (tid < G * w) {
        const int c = k + tid % w;
        for (int lr = lr0 + tid / w; lr < nr; lr += G)
          sacc = fma(P[lr * QNBP + k], P[lr * QNBP + c], sacc);
      }
      red[tid] = sacc;
      __syncthreads();
      if (tid < w) {
        double t = 0.0;
        for (int g = 0; g < G; g++) t += red[g * w + tid];
        mine[tid] = t;
      }
      __syncthreads();
    }
    for (int idx = tid; idx < w * CL; idx += QPT) {
      const int c = idx % w, dst = idx / w;
      st_remote_f64(remote_addr(&xch[par][rank][c], (uint32_t)dst), mine[c]);
    }
    const bool owner = jc >= r0 && jc < r0 + nr;
    if (owner)
      for (int idx = tid; idx < w * CL; idx += QPT) {
        const int c = idx % w, dst = idx / w;
        st_remote_f64(remote_addr(&own[par][c], (uint32_t)dst), P[(jc - r0) * QNBP + k + c]);
      }
    cluster_sync();
    // identical in every CTA: the sums in rank order, a, u0 and the factors
    if (tid < w) {
      double t = 0.0;
      for (int q = 0; q < CL; q++) t += xch[par][q][tid];
      tot[tid] = t;
    }
    __syncthreads();
    const double q = own[par][0];
    const double a = q > 0.0 ? -sqrt(tot[0]) : sqrt(tot[0]);
    const double u0 = q - a;
    if (a != 0.0 && tid > 0 && tid < w) fac[tid] = (tot[tid] - a * own[par][tid]) / (a * u0);
    if (rank == 0 && tid == 0) {
      p.rdiag[jc] = a;
      p.tau[k] = a != 0.0 ? -1.0 / (a * u0) : 0.0;
    }
    __syncthreads();
    if (a != 0.0 && w > 1) {  // columns k+1..nb-1, the same mapping
      const int w1 = w - 1, G = QPT / w1;
      if (tid < G * w1) {
        const int c = k + 1 + tid % w1;
        const double f = fac[c - k];
        for (int lr = lr0 + tid / w1; lr < nr; lr += G) {
          const double u = (r0 + lr == jc) ? u0 : P[lr * QNBP + k];
          P[lr * QNBP + c] = fma(f, u, P[lr * QNBP + c]);
        }
      }
    }
    if (a != 0.0 && owner && tid == 0) P[(jc - r0) * QNBP + k] = u0;
    __syncthreads();
  }
  // No remote access follows the last cluster barrier.
  for (int idx = tid; idx < nr * nb; idx += QPT) {
    const int lr = idx / nb, c = idx % nb;
    const int i = r0 + lr - p.j;
    const double v = P[lr * QNBP + c];
    if (i < nb) p.rsave[i * QB + c] = v;
    p.A[(size_t)(r0 + lr) * p.ld + p.j + c] = c > i ? 0.0 : v;
  }
  for (int idx = tid; idx < nr * nb; idx += QPT) {
    const int c = idx / nr, lr = idx % nr;
    const int i = r0 + lr - p.j;
    p.vt[(size_t)c * p.ldv + i] = c > i ? 0.0 : P[lr * QNBP + c];
  }
}

// out[r][c] = sum over z < splits of part[z][r][c] (ascending z).
__global__ void qr_wsum_kernel(const double* __restrict__ part, size_t ldp, size_t pzs, int splits,
                               int rows, int cols, double* __restrict__ out, size_t ldo) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)rows * cols) return;
  const int r = (int)(idx / cols), c = (int)(idx % cols);
  const double* src = part + (size_t)r * ldp + c;
  double s = 0.0;
  for (int z = 0; z < splits; z++) s += src[(size_t)z * pzs];
  out[(size_t)r * ldo + c] = s;
}

// W2[:, c] = T' W[:, c] (forward) or T W[:, c] (backward) for c < ncols, with
// T^-1 = diag(1/tau) + strictly_upper(G) (nb x nb, pitch ldg): one warp per
// column, lane l holding rows l and l + 32. Each step takes W2_i from its
// lane (a shuffle) and applies it to the rows still open (right-looking), so
// the chain per column is nb shuffles, with the FMAs of a step independent.
// gsave (when not null) receives G (pitch QB) from CTA 0.
__global__ void __launch_bounds__(QTS_W * 32)
qr_tsolve_kernel(const double* __restrict__ G, size_t ldg, const double* __restrict__ tau, int nb,
                 const double* __restrict__ W, size_t ldw, int ncols, double* __restrict__ W2,
                 size_t ldw2, int forward, double* __restrict__ gsave) {
  __shared__ double Gs[QB][QNBP];
  __shared__ double ts[QB];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int idx = tid; idx < nb * nb; idx += QTS_W * 32) {
    const int r = idx / nb, q = idx % nb;
    const double g = G[(size_t)r * ldg + q];
    Gs[r][q] = g;
    if (gsave && blockIdx.x == 0) gsave[r * QB + q] = g;
  }
  if (tid < QB) ts[tid] = tid < nb ? tau[tid] : 0.0;
  __syncthreads();
  const int c = blockIdx.x * QTS_W + warp;
  if (c >= ncols) return;
  const int r0 = lane, r1 = lane + 32;
  double a0 = r0 < nb ? W[(size_t)r0 * ldw + c] : 0.0;
  double a1 = r1 < nb ? W[(size_t)r1 * ldw + c] : 0.0;
  if (forward) {
    for (int i = 0; i < nb; i++) {
      const double v = ts[i] * __shfl_sync(0xffffffffu, i < 32 ? a0 : a1, i & 31);
      if (lane == (i & 31)) {
        if (i < 32) a0 = v; else a1 = v;
      }
      if (r0 > i && r0 < nb) a0 = fma(-Gs[i][r0], v, a0);
      if (r1 > i && r1 < nb) a1 = fma(-Gs[i][r1], v, a1);
    }
  } else {
    for (int i = nb - 1; i >= 0; i--) {
      const double v = ts[i] * __shfl_sync(0xffffffffu, i < 32 ? a0 : a1, i & 31);
      if (lane == (i & 31)) {
        if (i < 32) a0 = v; else a1 = v;
      }
      if (r0 < i) a0 = fma(-Gs[r0][i], v, a0);
      if (r1 < i) a1 = fma(-Gs[r1][i], v, a1);
    }
  }
  if (r0 < nb) W2[(size_t)r0 * ldw2 + c] = a0;
  if (r1 < nb) W2[(size_t)r1 * ldw2 + c] = a1;
}

// V of a factored block (rows [j, m), columns [j, j + nb)) in explicit form:
// vx (rows x QB) and vt (nb x rows, pitch ldv), zeros above the diagonal; and
// tau for get_q (mode 1) or solve (mode 2).
__global__ void qr_build_v_kernel(const double* __restrict__ A, size_t ld, int m, int j, int nb,
                                  const double* __restrict__ rdiag, int mode,
                                  double* __restrict__ vx, double* __restrict__ vt, size_t ldv,
                                  double* __restrict__ tau) {
  const int rows = m - j;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < (size_t)nb) {
    const int c = (int)idx;
    const double u0 = A[(size_t)(j + c) * ld + j + c];
    tau[c] = mode == 1 ? (u0 == 0.0 ? 0.0 : -1.0 / (rdiag[j + c] * u0)) : 1.0 / u0;
  }
  if (idx >= (size_t)rows * nb) return;
  const int i = (int)(idx / nb), c = (int)(idx % nb);
  const double v = c > i ? 0.0 : A[(size_t)(j + i) * ld + j + c];
  vx[(size_t)i * QB + c] = v;
  vt[(size_t)c * ldv + i] = v;
}

int blocks_of(size_t total, int t) { return (int)((total + t - 1) / t); }

// Cluster size (16, 8, or 0: no cluster launch) and the largest rows per CTA,
// once per device.
struct PanelCaps {
  int cluster;
  int rpc_max;
};
PanelCaps panel_caps(la_ctx ctx) {
  static PanelCaps caps_of[LA_MAX_DEVICES];
  static la_device_once once;
  const int dev = la_current_device();
  if (dev < 0 || dev >= LA_MAX_DEVICES) return {0, 0};
  const size_t optin = ctx->smem_optin;
  once.run([optin](int d) {
    PanelCaps c = {0, 0};
    cudaFuncAttributes fa;
    size_t stat = 0;
    if (cudaFuncGetAttributes(&fa, qr_panel_kernel) == cudaSuccess) stat = fa.sharedSizeBytes;
    const size_t dyn = optin > stat + 1024 ? optin - stat - 1024 : 0;
    const int rpc = (int)(dyn / (QNBP * sizeof(double)));
    if (rpc >= QB &&
        cudaFuncSetAttribute(qr_panel_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess &&
        cudaFuncSetAttribute(qr_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(rpc * QNBP * sizeof(double))) == cudaSuccess) {
      for (int cl : {16, 8}) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(cl);
        cfg.blockDim = dim3(QPT);
        cfg.dynamicSmemBytes = rpc * QNBP * sizeof(double);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cl;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, qr_panel_kernel, &cfg) == cudaSuccess && n >= 1) {
          c = {cl, rpc};
          break;
        }
      }
    }
    cudaGetLastError();
    caps_of[d] = c;
    return cudaSuccess;
  });
  return caps_of[dev];
}

la_status launch_qr_panel(la_ctx ctx, const QrPanelArgs& a, int cluster, cudaStream_t stream) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster);
  cfg.blockDim = dim3(QPT);
  cfg.dynamicSmemBytes = (size_t)a.rpc * QNBP * sizeof(double);
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, qr_panel_kernel, a);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaLaunchKernelEx(qr_panel)");
  ctx->launches++;
  return LA_OK;
}

// Split of the K = rows inner products over `tiles` output tiles: enough
// pieces for about three CTAs per SM, each at least two 32-deep slabs.
void split_plan(la_ctx ctx, int tiles, int K, int* splits, int* kper) {
  const int target = 3 * std::max(1, ctx->sm_count);
  int s = std::max(1, std::min(std::max(1, K / 64), target / std::max(1, tiles)));
  int kp = (K + s - 1) / s;
  kp = std::max(32, (kp + 31) / 32 * 32);
  *kper = kp;
  *splits = std::max(1, (K + kp - 1) / kp);
}

size_t pad4b(size_t x) { return (x + 3) & ~size_t(3); }

struct DevBuf {
  la_ctx ctx;
  void* p = nullptr;
  explicit DevBuf(la_ctx c) : ctx(c) {}
  ~DevBuf() { la_device_free(ctx, p); }
  la_status alloc(size_t doubles) { return la_device_alloc(ctx, &p, doubles * sizeof(double)); }
  double* d() const { return static_cast<double*>(p); }
};

// W = V' T[j:, cols] (nb x ncols) by split-K GEMM and reduction into wf
// (pitch ldw), from vt (nb x rows, pitch ldv) and T (pitch ldt).
la_status apply_vt(la_ctx ctx, const double* vt, size_t ldv, int nb, int rows, const double* T,
                   size_t ldt, int ncols, double* part, size_t part_cap, double* wf, size_t ldw) {
  int splits, kper;
  split_plan(ctx, (ncols + 63) / 64, rows, &splits, &kper);
  const size_t ldp = pad4b((size_t)ncols), pzs = (size_t)nb * ldp;
  if ((size_t)splits * pzs > part_cap) return LA_INVALID;
  LA_TRY(launch_gemm_splitk(ctx, nb, ncols, rows, vt, ldv, T, ldt, part, ldp, pzs, splits, kper));
  const size_t total = (size_t)nb * ncols;
  qr_wsum_kernel<<<blocks_of(total, 256), 256, 0, ctx->stream>>>(part, ldp, pzs, splits, nb, ncols,
                                                                wf, ldw);
  ctx->launches++;
  return la_check_launch(ctx, "qr_wsum_kernel");
}

la_status launch_tsolve(la_ctx ctx, const double* G, size_t ldg, const double* tau, int nb,
                        const double* W, size_t ldw, int ncols, double* W2, size_t ldw2,
                        bool forward, double* gsave) {
  if (ncols <= 0 && !gsave) return LA_OK;
  qr_tsolve_kernel<<<std::max(1, blocks_of((size_t)std::max(ncols, 0), QTS_W)), QTS_W * 32, 0,
                     ctx->stream>>>(G, ldg, tau, nb, W, ldw, std::max(ncols, 0), W2, ldw2,
                                    forward ? 1 : 0, gsave);
  ctx->launches++;
  return la_check_launch(ctx, "qr_tsolve_kernel");
}

// The largest partial-product buffer over the blocks: splits x nb x pitch.
size_t part_doubles(la_ctx ctx, int m, int dc, int cols_total, bool cols_from_j) {
  size_t cap = 0;
  for (int j = 0; j < dc; j += QB) {
    const int ncols = cols_from_j ? cols_total - j : cols_total;
    if (ncols <= 0) continue;
    int splits, kper;
    split_plan(ctx, (ncols + 63) / 64, m - j, &splits, &kper);
    cap = std::max(cap, (size_t)splits * QB * pad4b((size_t)ncols));
  }
  return cap;
}

}  // namespace

bool qr_blocked_supported(la_ctx ctx, int m, int n) {
  const int dc = std::min(m, n);
  if (dc < 2 * QB) return false;
  const PanelCaps c = panel_caps(ctx);
  if (c.cluster == 0) return false;
  return (m + c.cluster - 1) / c.cluster <= c.rpc_max;
}

la_status qr_blocked_factor(la_ctx ctx, double* A, size_t ld, int m, int n, double* rdiag,
                            double* gram) {
  const int dc = std::min(m, n);
  const PanelCaps caps = panel_caps(ctx);
  if (caps.cluster == 0 || (m + caps.cluster - 1) / caps.cluster > caps.rpc_max)
    return LA_UNSUPPORTED;
  const size_t ldv = pad4b((size_t)m), ldw = pad4b((size_t)n);
  const size_t pcap = part_doubles(ctx, m, dc, n, true);
  DevBuf vt(ctx), rsave(ctx), tau(ctx), part(ctx), wf(ctx), w2(ctx);
  LA_TRY(vt.alloc((size_t)QB * ldv));
  LA_TRY(rsave.alloc((size_t)2 * QB * QB));  // alternating by block parity
  LA_TRY(tau.alloc(QB));
  LA_TRY(part.alloc(std::max<size_t>(pcap, 1)));
  LA_TRY(wf.alloc((size_t)QB * ldw));
  LA_TRY(w2.alloc((size_t)QB * ldw));
  cudaStream_t ms = ctx->stream;
  const bool look = ctx->lookahead != 0 && ctx->side_stream != nullptr;
  auto panel = [&](int b, cudaStream_t s) {
    const int j = b * QB;
    QrPanelArgs a;
    a.A = A;
    a.ld = ld;
    a.m = m;
    a.j = j;
    a.nb = std::min(QB, dc - j);
    a.rpc = (m - j + caps.cluster - 1) / caps.cluster;
    a.rdiag = rdiag;
    a.tau = tau.d();
    a.vt = vt.d();
    a.ldv = ldv;
    a.rsave = rsave.d() + (size_t)(b & 1) * QB * QB;
    return launch_qr_panel(ctx, a, caps.cluster, s);
  };
  // Lookahead (as in the mixed LU): once the next block's columns are
  // updated, its panel runs on the side stream beside the update of the rest.
  // The two touch disjoint columns; tau and V' are consumed before the fork
  // and the top squares' saved content alternates between two buffers.
  LA_TRY(panel(0, ms));
  bool forked = false;
  for (int j = 0, b = 0; j < dc; j += QB, b++) {
    const int nb = std::min(QB, dc - j), rows = m - j, ncols = n - j;
    const int nbn = j + nb < dc ? std::min(QB, dc - j - nb) : 0;  // the next block's width
    double* Aj = A + (size_t)j * ld + j;
    if (forked) {
      LA_CUDA(ctx, cudaStreamWaitEvent(ms, ctx->ev_join, 0));
      forked = false;
    }
    // [G | W] = V' A[j:, j:]
    LA_TRY(apply_vt(ctx, vt.d(), ldv, nb, rows, Aj, ld, ncols, part.d(), pcap, wf.d(), ldw));
    // W2 = T' W for the columns right of the block; G kept for get_q and solve
    LA_TRY(launch_tsolve(ctx, wf.d(), ldw, tau.d(), nb, wf.d() + nb, ldw, ncols - nb, w2.d(), ldw,
                         true, gram + (size_t)b * QB * QB));
    // A[j:, j+nb:] -= V W2: the next block's columns first when it runs ahead
    // (an odd width would misalign the rest's operand: no split then)
    const bool split = look && nbn > 0 && nbn % 2 == 0 && ncols - nb > nbn;
    if (split) {
      LA_TRY(launch_gemm(ctx, GM_FMA_SUB, rows, nbn, nb, Aj, ld, w2.d(), ldw, Aj + nb, ld));
      LA_CUDA(ctx, cudaEventRecord(ctx->ev_fork, ms));
      LA_CUDA(ctx, cudaStreamWaitEvent(ctx->side_stream, ctx->ev_fork, 0));
      LA_TRY(panel(b + 1, ctx->side_stream));
      LA_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->side_stream));
      forked = true;
      LA_TRY(launch_gemm(ctx, GM_FMA_SUB, rows, ncols - nb - nbn, nb, Aj, ld, w2.d() + nbn, ldw,
                         Aj + nb + nbn, ld));
    } else {
      if (ncols > nb)
        LA_TRY(launch_gemm(ctx, GM_FMA_SUB, rows, ncols - nb, nb, Aj, ld, w2.d(), ldw, Aj + nb, ld));
    }
    LA_TRY(launch_copy2d(ctx, rsave.d() + (size_t)(b & 1) * QB * QB, QB, Aj, ld, nb, nb));
    if (!split && nbn > 0) LA_TRY(panel(b + 1, ms));
  }
  if (forked) LA_CUDA(ctx, cudaStreamWaitEvent(ms, ctx->ev_join, 0));
  return LA_OK;
}

la_status qr_blocked_apply(la_ctx ctx, const double* A, size_t ld, int m, int dc,
                           const double* rdiag, const double* gram, int mode, double* T,
                           size_t ldt, int cols) {
  const bool getq = mode == 1;
  const size_t ldv = pad4b((size_t)m), ldw = pad4b((size_t)cols);
  const size_t pcap = part_doubles(ctx, m, dc, cols, getq);
  DevBuf vx(ctx), vt(ctx), tau(ctx), part(ctx), wf(ctx), w2(ctx);
  LA_TRY(vx.alloc((size_t)m * QB));
  LA_TRY(vt.alloc((size_t)QB * ldv));
  LA_TRY(tau.alloc(QB));
  LA_TRY(part.alloc(std::max<size_t>(pcap, 1)));
  LA_TRY(wf.alloc((size_t)QB * ldw));
  LA_TRY(w2.alloc((size_t)QB * ldw));
  const int nblocks = (dc + QB - 1) / QB;
  for (int s = 0; s < nblocks; s++) {
    const int b = getq ? nblocks - 1 - s : s;
    const int j = b * QB, nb = std::min(QB, dc - j), rows = m - j;
    const int c0 = getq ? j : 0, ncols = cols - c0;
    qr_build_v_kernel<<<blocks_of((size_t)rows * nb, 256), 256, 0, ctx->stream>>>(
        A, ld, m, j, nb, rdiag, mode, vx.d(), vt.d(), ldv, tau.d());
    ctx->launches++;
    LA_TRY(la_check_launch(ctx, "qr_build_v_kernel"));
    double* Tj = T + (size_t)j * ldt + c0;
    LA_TRY(apply_vt(ctx, vt.d(), ldv, nb, rows, Tj, ldt, ncols, part.d(), pcap, wf.d(), ldw));
    LA_TRY(launch_tsolve(ctx, gram + (size_t)b * QB * QB, QB, tau.d(), nb, wf.d(), ldw, ncols,
                         w2.d(), ldw, !getq, nullptr));
    LA_TRY(launch_gemm(ctx, GM_FMA_SUB, rows, ncols, nb, vx.d(), QB, w2.d(), ldw, Tj, ldt));
  }
  return LA_OK;
}
