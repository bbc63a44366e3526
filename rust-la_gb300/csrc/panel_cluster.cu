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
//
// panel_cluster_reg_kernel (used when each thread holds at most 4 rows) keeps
// the rows in registers instead: thread t of CTA g owns rows row0 + t + 256 q
// with their 32 panel values and their current positions. Rows never move
// between threads; a pivot exchange swaps two position registers, and each
// row is written to its final position at the end. With up to 2 rows per
// thread each row's registers rotate left by one slot per column, so the
// current column is always slot 0 and the update is 31 FMAs with fixed
// register indices; the finished values collect at the end of the window, and
// the published pivot row carries zeros there so that the update leaves them
// unchanged. The column loop is not unrolled (an unrolled 32-column body with
// 4 rows per thread outgrew the instruction cache), and the pivot row streams
// from shared memory into the update. Per column: the warp's
// best (key, position) is one 64-bit word (key high, bit-inverted position
// low, so the integer maximum is the reference's first maximum), the winning
// lane of each warp publishes its row, one CTA barrier, and warp 0 pushes the
// CTA's candidate (key and row, 144 bytes) into slot g of every CTA's receive
// buffer with st.async, which completes the bytes on the receiving CTA's
// mbarrier. Each CTA waits on its own mbarrier for the C candidates (bounded)
// and then reads the winner's row locally. The receive buffers and barriers
// alternate by column parity; a CTA can push column c + 2 only after every
// CTA has pushed column c + 1, which each does after reading its column-c
// slots, so no slot is overwritten before it is read. Cluster barriers remain
// only at the start (barriers initialised) and the end (no CTA leaves while
// pushes into it may be in flight).
#include "la_internal.cuh"
#include "swap_compose.cuh"

namespace {

constexpr int CW = 32;      // panel width
constexpr int CP = CW + 1;  // padded row pitch in shared memory
constexpr int CT = 256;     // threads per CTA
constexpr int PNW = CT / 32;  // warps per CTA
constexpr int PSLOT = 36;     // words per pushed candidate: key (2), padding (2), row (32)

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
  int* err;  // the context's error word (bounded waits)
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
  __shared__ int s_atp[SWAP_SLOTS], s_atr[SWAP_SLOTS];
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
  if (g == 0 && warp == 0)
    compose_swaps_warp(s_pivs, jb, p.j0, false, nullptr, p.swaps, s_atp, s_atr, lane);
}

__device__ __forceinline__ unsigned long long gtimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Wait for the phase `parity` of a local mbarrier that remote CTAs complete
// (acquire at cluster scope); gives up after 2 s or when the error word is
// set, recording DERR_PANEL_TIMEOUT.
__device__ bool cluster_mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(bar));
  unsigned long long t0 = 0;
  for (unsigned i = 0;; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 63u) == 63u) {
      if (*reinterpret_cast<volatile int*>(err) != 0) return false;
      const unsigned long long now = gtimer_ns();
      if (t0 == 0) t0 = now;
      else if (now - t0 > 2000000000ull) {
        atomicCAS(err, 0, (int)DERR_PANEL_TIMEOUT);
        return false;
      }
    }
  }
}
// 16-byte asynchronous store into another CTA's shared memory that completes
// `bytes` on that CTA's mbarrier (both addresses from mapa).
__device__ __forceinline__ void st_async_v4(uint32_t dst, uint32_t bar, uint32_t x, uint32_t y,
                                            uint32_t z, uint32_t w) {
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::
          "r"(dst), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
      : "memory");
}

// Largest 64-bit value over the full warp (every lane gets it), as two 32-bit
// warp reductions (redux.sync): the high words, then the low words of the
// lanes whose high word is the largest; shorter than five rounds of 64-bit
// shuffles on the column's critical path.
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long x) {
  const unsigned hi = (unsigned)(x >> 32), lo = (unsigned)x;
  const unsigned mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? lo : 0u);
  return ((unsigned long long)mh << 32) | ml;
}

// One column of panel_cluster_reg_kernel (see there); false when a wait gave
// up. The rows' register windows rotate: columns are taken in pairs, the
// first at slot S = 0 and the second at slot S = 1, and each window moves by
// two slots after the pair (ROT = 2); a lone last column uses S = 0, ROT = 1.
// So the window stays put within a pair and moves by two instead of twice by
// one. Slot k of the window at S = 1 is slot k - 1 of the window the pair's
// first column would have left after a one-slot move, so every column meets
// the same values in the same operations.
template <int RPT, int S, int ROT>
__device__ __forceinline__ bool panel_column(int c, const ClusterPanelArgs& p, int g, int C,
                                             int tid, int lane, int warp, float (&v)[RPT][CW],
                                             int (&pos)[RPT], float (*wrow)[PNW][CW],
                                             unsigned long long (*wkey)[PNW],
                                             uint32_t (*recv)[16][PSLOT], uint64_t* rbar,
                                             int* s_pivs) {
  constexpr int NW = PNW;
  constexpr uint32_t SLOT_BYTES = PSLOT * 4;
    const int j = p.j0 + c, par = c & 1;
    // 1. this thread's and this warp's best candidate
    unsigned long long best = 0ull;
    int bq = 0;
#pragma unroll
    for (int q = 0; q < RPT; q++)
      if (pos[q] >= j) {
        const unsigned long long pk =
            ((unsigned long long)ckey(v[q][S], pos[q], j) << 32) |
            (unsigned)(~pos[q]);
        if (pk > best) { best = pk; bq = q; }
      }
    const unsigned long long wb = warp_max_u64(best);
    const unsigned wmask = __ballot_sync(0xffffffffu, wb != 0ull && best == wb);
    if (wmask && lane == __ffs(wmask) - 1) {
      // published without its finished slots (zeros: the update leaves the
      // other rows' finished slots as they are)
      float* dst = wrow[par][warp];
#pragma unroll
      for (int q = 0; q < RPT; q++)
        if (q == bq) {
#pragma unroll
          for (int k = 0; k < CW; k++) dst[k] = (k >= S && k < S + CW - c) ? v[q][k] : 0.f;
        }
    }
    if (lane == 0) wkey[par][warp] = wb;
    __syncthreads();
    // 2. warp 0 pushes the CTA's candidate (key and row) into slot g of every
    //    CTA's receive buffer (the slots alternate by column parity).
    if (warp == 0) {
      const unsigned long long k = lane < NW ? wkey[par][lane] : 0ull;
      const unsigned long long km = warp_max_u64(k);
      const unsigned cm = __ballot_sync(0xffffffffu, km != 0ull && k == km);
      const float* crow = wrow[par][cm ? __ffs(cm) - 1 : 0];
      if (lane < C) {
        const uint32_t dst = remote_addr(&recv[par][g][0], (uint32_t)lane);
        const uint32_t bar = remote_addr(&rbar[par], (uint32_t)lane);
        st_async_v4(dst, bar, (uint32_t)km, (uint32_t)(km >> 32), 0u, 0u);
#pragma unroll
        for (int q = 0; q < CW / 4; q++) {
          const float4 t = reinterpret_cast<const float4*>(crow)[q];
          st_async_v4(dst + 16 + 16 * q, bar, __float_as_uint(t.x), __float_as_uint(t.y),
                      __float_as_uint(t.z), __float_as_uint(t.w));
        }
      }
      if (lane == 0)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                         static_cast<uint32_t>(__cvta_generic_to_shared(&rbar[par]))),
                     "r"((uint32_t)C * SLOT_BYTES)
                     : "memory");
    }
    // 3. every CTA's candidate has landed here (or the wait gave up)
    const bool got = cluster_mbar_wait(&rbar[par], (uint32_t)((c >> 1) & 1), p.err);
    if (!__syncthreads_and(got ? 1 : 0)) return false;
    // 4. the winner and its row, from local shared memory
    const unsigned long long gk =
        lane < C ? *reinterpret_cast<const unsigned long long*>(&recv[par][lane][0]) : 0ull;
    const unsigned long long gm = warp_max_u64(gk);
    const unsigned gmask = __ballot_sync(0xffffffffu, lane < C && gk == gm);
    const int gsrc = __ffs(gmask) - 1;  // the row at position j is a candidate: gm != 0
    const int piv = (int)(~(unsigned)(gm & 0xffffffffull));
    const float* urow = reinterpret_cast<const float*>(&recv[par][gsrc][4]);
    {
      // The pivot row streams from shared memory in float4 chunks, each chunk
      // applied to all of this thread's rows (4 registers for it, not 32).
      const float d = urow[S];
      const float sc = d != 0.f ? 1.f / d : 1.f;
      float lq[RPT];
      bool act[RPT];
#pragma unroll
      for (int q = 0; q < RPT; q++) {
        act[q] = false;
        if (pos[q] == piv) {
          pos[q] = j;  // the pivot row; it keeps its values
        } else {
          if (pos[q] == j) pos[q] = piv;  // the displaced row takes the pivot's place
          act[q] = pos[q] > j;
        }
        lq[q] = d != 0.f ? v[q][S] * sc : v[q][S];
        if (act[q]) v[q][S] = lq[q];
      }
#pragma unroll
      for (int k4 = 0; k4 < CW / 4; k4++) {
        const float4 u4 = reinterpret_cast<const float4*>(urow)[k4];
        const float uk[4] = {u4.x, u4.y, u4.z, u4.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int k = 4 * k4 + i;
          if (k == S) continue;
#pragma unroll
          for (int q = 0; q < RPT; q++)
            if (act[q]) v[q][k] = fmaf(-lq[q], uk[i], v[q][k]);
        }
      }
#pragma unroll
      for (int q = 0; q < RPT; q++) {
        // rotate by ROT: the next column comes to slot 0, the finished values
        // to the end
        float t[ROT > 0 ? ROT : 1];
#pragma unroll
        for (int r = 0; r < ROT; r++) t[r] = v[q][r];
#pragma unroll
        for (int k = 0; k < CW - ROT; k++) v[q][k] = v[q][k + ROT];
#pragma unroll
        for (int r = 0; r < ROT; r++) v[q][CW - ROT + r] = t[r];
      }
      if (g == 0 && tid == 0) {
        p.ipiv[j] = piv;
        s_pivs[c] = piv;
      }
    }
  return true;
}

template <int RPT>
__global__ void __launch_bounds__(CT, 1) panel_cluster_reg_kernel(ClusterPanelArgs p) {
  la_pdl_wait();
  la_pdl_trigger();
  __shared__ __align__(16) float wrow[2][PNW][CW];
  __shared__ unsigned long long wkey[2][PNW];
  __shared__ __align__(16) uint32_t recv[2][16][PSLOT];
  __shared__ __align__(8) uint64_t rbar[2];
  __shared__ int s_pivs[CW];
  __shared__ int s_atp[SWAP_SLOTS], s_atr[SWAP_SLOTS];

  const int g = (int)cta_rank();
  const int C = (int)gridDim.x;  // one cluster per launch, C <= 16
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int rpc = p.rpc, jb = p.jb;
  const int row0 = p.j0 + g * rpc;
  const int nrows = max(0, min(rpc, p.m - row0));
  const bool vec = (p.ld % 4 == 0) && (p.j0 % 4 == 0) &&
                   (reinterpret_cast<uintptr_t>(p.A) % 16 == 0);

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(&rbar[0]))));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                     static_cast<uint32_t>(__cvta_generic_to_shared(&rbar[1]))));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  float v[RPT][CW];
  int pos[RPT];
#pragma unroll
  for (int q = 0; q < RPT; q++) {
    const int lr = q * CT + tid;
    pos[q] = lr < nrows ? row0 + lr : -1;
    const float* src = p.A + (size_t)(lr < nrows ? row0 + lr : 0) * p.ld + p.j0;
    if (pos[q] >= 0 && vec && jb == CW) {
#pragma unroll
      for (int c4 = 0; c4 < CW / 4; c4++) {
        const float4 t = reinterpret_cast<const float4*>(src)[c4];
        v[q][4 * c4] = t.x;
        v[q][4 * c4 + 1] = t.y;
        v[q][4 * c4 + 2] = t.z;
        v[q][4 * c4 + 3] = t.w;
      }
    } else {
#pragma unroll
      for (int c = 0; c < CW; c++) v[q][c] = (pos[q] >= 0 && c < jb) ? src[c] : 0.f;
    }
  }
  cluster_sync();  // every CTA's receive barriers are initialised before any push

  // The register windows rotate for every row count: an unrolled 32-column
  // body with static register indices (4 rows per thread) outgrew the
  // instruction cache and stalled on instruction fetch; the rotating loop
  // stays in cache even where it spills a little at 4 rows per thread.
  bool ok = true;
  for (int c = 0; c < jb && ok; c += 2) {
    if (c + 1 < jb) {
      ok = panel_column<RPT, 0, 0>(c, p, g, C, tid, lane, warp, v, pos, wrow, wkey, recv, rbar,
                                   s_pivs) &&
           panel_column<RPT, 1, 2>(c + 1, p, g, C, tid, lane, warp, v, pos, wrow, wkey, recv,
                                   rbar, s_pivs);
    } else {
      ok = panel_column<RPT, 0, 1>(c, p, g, C, tid, lane, warp, v, pos, wrow, wkey, recv, rbar,
                                   s_pivs);
    }
  }
  cluster_sync();  // no CTA leaves while pushes into its shared memory may be in flight
  if (!ok) return;
  // jb rotations so far; 32 in all bring every value back to its column
  for (int r = jb; r < CW; r++)
#pragma unroll
    for (int q = 0; q < RPT; q++) {
      const float t = v[q][0];
#pragma unroll
      for (int k = 0; k < CW - 1; k++) v[q][k] = v[q][k + 1];
      v[q][CW - 1] = t;
    }

  // each row to its final position
#pragma unroll
  for (int q = 0; q < RPT; q++)
    if (pos[q] >= 0) {
      float* dst = p.A + (size_t)pos[q] * p.ld + p.j0;
      if (vec && jb == CW) {
#pragma unroll
        for (int c4 = 0; c4 < CW / 4; c4++)
          reinterpret_cast<float4*>(dst)[c4] =
              make_float4(v[q][4 * c4], v[q][4 * c4 + 1], v[q][4 * c4 + 2], v[q][4 * c4 + 3]);
      } else {
#pragma unroll
        for (int c = 0; c < CW; c++)
          if (c < jb) dst[c] = v[q][c];
      }
    }
  if (g == 0 && warp == 0)
    compose_swaps_warp(s_pivs, jb, p.j0, false, nullptr, p.swaps, s_atp, s_atr, lane);
}


}  // namespace

// Launches panel_cluster_reg_kernel<RPT> as one cluster of `cluster` CTAs;
// LA_UNSUPPORTED (nothing launched) when such a cluster cannot be resident.
template <int RPT>
la_status launch_reg(la_ctx ctx, float* A, size_t ld, int m, int j0, int jb, int* d_ipiv,
                     int cluster, int rpc) {
  // Cluster size checked once per instantiation and device (0: none).
  static int ok_for[LA_MAX_DEVICES];
  static la_device_once once;
  const int dev = la_current_device();
  if (dev < 0 || dev >= LA_MAX_DEVICES) return LA_UNSUPPORTED;
  once.run([cluster](int d) {
    ok_for[d] = 0;
    if (cudaFuncSetAttribute(panel_cluster_reg_kernel<RPT>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(cluster);
      cfg.blockDim = dim3(CT);
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = cluster;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, panel_cluster_reg_kernel<RPT>, &cfg) ==
              cudaSuccess &&
          nclusters >= 1)
        ok_for[d] = cluster;
    }
    cudaGetLastError();
    return cudaSuccess;
  });
  if (ok_for[dev] != cluster) return LA_UNSUPPORTED;
  ClusterPanelArgs a;
  a.A = A;
  a.ld = ld;
  a.m = m;
  a.j0 = j0;
  a.jb = jb;
  a.rpc = rpc;
  a.ipiv = d_ipiv;
  a.swaps = ctx->d_swaps;
  a.err = ctx->d_err;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cluster);
  cfg.blockDim = dim3(CT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = ctx->pdl_now ? 2 : 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, panel_cluster_reg_kernel<RPT>, a);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaLaunchKernelEx(panel_cluster_reg)");
  ctx->launches++;
  return LA_OK;
}


// Returns LA_UNSUPPORTED (without launching) when the panel does not fit one
// cluster; the caller then uses the cooperative kernel.
la_status launch_panel_cluster_f32(la_ctx ctx, float* A, size_t ld, int m, int j0, int jb,
                                   int* d_ipiv) {
  const int R = m - j0;
  if (R <= 0 || jb <= 0) return LA_OK;
  if (jb > CW) return LA_UNSUPPORTED;
  // Per device: the cluster size (16, 8 or 0 = no cluster launch possible)
  // and the dynamic shared memory the cluster kernel may use.
  static int cluster_of[LA_MAX_DEVICES];
  static size_t max_smem_of[LA_MAX_DEVICES];
  static la_device_once once;
  const int dev = la_current_device();
  if (dev < 0 || dev >= LA_MAX_DEVICES) return LA_UNSUPPORTED;
  const size_t optin = ctx->smem_optin;
  once.run([optin](int d) {
    int cl = 0;
    size_t ms = optin - 2048;  // room for the static buffers
    if (cudaFuncSetAttribute(panel_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed,
                             1) != cudaSuccess ||
        cudaFuncSetAttribute(panel_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)ms) != cudaSuccess) {
      cudaGetLastError();
      ms = 0;
    }
    for (int c : {16, 8}) {
      if (ms == 0) break;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(c);
      cfg.blockDim = dim3(CT);
      cfg.dynamicSmemBytes = ms;
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
        cl = c;
        break;
      }
      cudaGetLastError();
    }
    cluster_of[d] = cl;
    max_smem_of[d] = ms;
    return cudaSuccess;
  });
  const int cluster = cluster_of[dev];
  const size_t max_smem = max_smem_of[dev];
  if (cluster == 0) return LA_UNSUPPORTED;
  const int rpc = (R + cluster - 1) / cluster;
  {
    // Register rows: at most 4 rows per thread.
    const int rpt = (rpc + CT - 1) / CT;
    la_status rs = LA_UNSUPPORTED;
    if (rpt <= 1) rs = launch_reg<1>(ctx, A, ld, m, j0, jb, d_ipiv, cluster, rpc);
    else if (rpt <= 2) rs = launch_reg<2>(ctx, A, ld, m, j0, jb, d_ipiv, cluster, rpc);
    else if (rpt <= 4) rs = launch_reg<4>(ctx, A, ld, m, j0, jb, d_ipiv, cluster, rpc);
    if (rs != LA_UNSUPPORTED) return rs;
  }
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
  a.err = ctx->d_err;
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
