// Batched solves of many small, unevenly sized systems (not in the reference;
// each system is LUDecomposition::new + solve, lu.rs:104-278, on its own).
//
// One persistent kernel per pass: every CTA takes the next system from an
// atomic work queue (descriptors sorted by decreasing n, i.e. by cost, so the
// largest systems start first and the tail is short), then
//   loads A_i (FP64 in HBM) into its working matrix: shared memory when the
//   system's whole layout fits the CTA's budget, else the CTA's slice of a
//   global scratch buffer;
//   factors it by a blocked right-looking LU with partial pivoting (the
//   reference's first-maximum pivot rule, lu.rs:132-137) with implicit row
//   swaps: a row map sends logical rows to physical rows, so a swap moves two
//   integers and the final map is the permutation P (lu.rs:245-254);
//   solves for B_i and writes X_i.
// Per 16-column panel: the panel is staged in shared memory in the arithmetic
// type, factored column by column (each thread owns rows, two barriers per
// column), written back; U12 = L11^-1 A12 is solved with each column in
// registers; A22 -= L21 U12 is register-tiled (a thread holds 4x4 of A22 and
// its rows of L21, all loads of a tile are issued before its FMAs).
// The working matrix is stored in the system's factor precision: FP64 (plain
// pass), FP32, BF16 or FP8 e4m3 (mixed pass; FP8 with a power-of-two scale of
// A_i), with FP32 arithmetic for the low precisions. Narrower storage keeps
// larger systems in shared memory but gives less accurate factors. The mixed
// pass then refines each system in FP64 (r = b - A x with A_i read again in
// FP64, d = LU \ r, x += d) until its normwise backward error <= tol or
// max_iters; systems that do not converge are flagged and the FP64 pass, run
// after it in the same CUDA graph, redoes only those. All state is per CTA; no
// CTA waits on another.
#include <cuda_fp8.h>

#include "f64conv.h"
#include "la_internal.cuh"

namespace {

constexpr int BT_MAX = 256;  // threads per CTA (one system per CTA): 64, 128 or 256
constexpr int NW_MAX = BT_MAX / 32;
constexpr int NMAX = 512;  // largest system
constexpr int PBW = 16;    // panel width of the per-system LU
constexpr int SP = 17;     // pitch of the staged panel (odd: rows fall in distinct banks)
constexpr int GM_M = 20;     // largest Krylov basis of one GMRES correction
constexpr int GM_OUTER = 2;  // GMRES-IR steps after LU-IR stalls
constexpr double GM_TOL = 1e-12;  // relative preconditioned residual of a GMRES correction
constexpr double GM_TRIGGER = 1e-6;  // LU-IR must have reached this backward error
// Hessenberg matrix [GM_M + 1][GM_M], right-hand side g, rotations cs, sn
constexpr size_t GM_SMALL = (size_t)((GM_M + 1) * GM_M + 3 * (GM_M + 1)) * sizeof(double);
// The Krylov basis lives in the CTA's global scratch slice, after the space of
// an FP32 working matrix of NMAX x NMAX.
constexpr size_t GM_V_OFFSET = (size_t)NMAX * NMAX * sizeof(float);

struct SysDesc {
  long long a;  // offset of A_i (n x n, row-major) in the A buffer, elements
  long long b;  // offset of B_i / X_i (n x nrhs, row-major), elements
  int n, nrhs, cls;
  int poff;     // offset of the system's row order in BatchArgs::piv
};

// Storage policies: element type in memory, arithmetic type, conversions.
struct StF64 {
  using S = double;
  using R = double;
  static __device__ __forceinline__ R ld(const S* p) { return *p; }
  static __device__ __forceinline__ S cv(R v) { return v; }
  static __device__ __forceinline__ R up(S v) { return v; }
};
struct StF32 {
  using S = float;
  using R = float;
  static __device__ __forceinline__ R ld(const S* p) { return *p; }
  static __device__ __forceinline__ S cv(R v) { return v; }
  static __device__ __forceinline__ R up(S v) { return v; }
};
struct StBF16 {
  using S = __nv_bfloat16;
  using R = float;
  static __device__ __forceinline__ R ld(const S* p) { return __bfloat162float(*p); }
  static __device__ __forceinline__ S cv(R v) { return __float2bfloat16_rn(v); }
  static __device__ __forceinline__ R up(S v) { return __bfloat162float(v); }
};
struct StFP8 {
  using S = __nv_fp8_e4m3;
  using R = float;
  static __device__ __forceinline__ R ld(const S* p) { return static_cast<float>(*p); }
  static __device__ __forceinline__ S cv(R v) { return __nv_fp8_e4m3(v); }
  static __device__ __forceinline__ R up(S v) { return static_cast<float>(v); }
};

template <typename R>
__device__ __forceinline__ unsigned long long bkey(R v, int pos, int j) {
  if (sizeof(R) == 8) {
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

struct Shared {
  // per-warp pivot candidates (key, logical position, staged row), by column parity
  unsigned long long rk[2][NW_MAX];
  int rp[2][NW_MAX];
  int rs[2][NW_MAX];
  // [0] ||A||_inf, [1 + c] max |r_c|, [5 + c] max |x_c|, [9 + c] max |b_c|,
  // [13] max |a_ij| (FP8 scaling)
  double norm[14];
  double red[NW_MAX];  // block reductions
  double gres;         // GMRES residual estimate (broadcast)
};

__host__ __device__ constexpr size_t al16(size_t x) { return (x + 15) / 16 * 16; }

// Shared-memory layout of one system (byte offsets into the dynamic shared
// memory): [M if resident][staged panel][U12][row map][x FP64][d FP32].
struct Lay {
  size_t stage, us, rmap, x, d, gm, total;
};
template <typename S, typename R>
__host__ __device__ Lay lay(int n, int nrhs, bool resident, bool mixed) {
  Lay L;
  size_t o = resident ? al16((size_t)n * n * sizeof(S)) : 0;
  L.stage = o;
  o += al16((size_t)n * SP * sizeof(R));
  L.us = o;
  o += al16((size_t)PBW * n * sizeof(R));
  L.rmap = o;  // rmap, then the panel's perm and spos (block_lu)
  o += al16((size_t)3 * n * sizeof(int));
  L.x = o;
  o += al16((size_t)n * nrhs * sizeof(double));
  L.d = o;
  o += mixed ? al16((size_t)n * nrhs * sizeof(float)) : 0;
  L.gm = o;  // GMRES: work vector w (n FP64), then the small arrays
  o += mixed ? al16((size_t)n * sizeof(double) + GM_SMALL) : 0;
  L.total = o;
  return L;
}

// A22 -= L21 U12 for the trailing nr x nr block (logical rows/columns >= j1):
// warp w, lane l computes rows rb + w + NW t (t < TR) and columns
// cb + l + 32 q (q < QN), with its L21 rows (staged rows perm[PBW + i]) in
// registers; all loads of a tile are issued before its FMAs. QN is picked
// from nr so that narrow trailing blocks do not run idle columns.
template <typename P, int TR, int QN>
__device__ __forceinline__ void trailing_update(typename P::S* M, int p, const int* rmap, int j1,
                                                int nr, const typename P::R* st,
                                                const typename P::R* us, const int* perm) {
  const int BT = blockDim.x, NW = BT >> 5;
  using S = typename P::S;
  using R = typename P::R;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int rb = 0; rb < nr; rb += NW * TR) {
    R lr[TR][PBW];
    S* crow[TR];
#pragma unroll
    for (int t = 0; t < TR; t++) {
      const int i = rb + warp + NW * t;
      const bool ok = i < nr;
      crow[t] = ok ? M + (size_t)rmap[j1 + i] * p + j1 : nullptr;
      const R* lrow = ok ? st + perm[PBW + i] * SP : st;
#pragma unroll
      for (int k = 0; k < PBW; k++) lr[t][k] = ok ? lrow[k] : R(0);
    }
    for (int cb = 0; cb < nr; cb += 32 * QN) {
      R acc[TR][QN];
#pragma unroll
      for (int t = 0; t < TR; t++)
#pragma unroll
        for (int q = 0; q < QN; q++) {
          const int c = cb + lane + 32 * q;
          acc[t][q] = (crow[t] && c < nr) ? P::ld(&crow[t][c]) : R(0);
        }
#pragma unroll
      for (int k = 0; k < PBW; k++) {
        R uv[QN];
#pragma unroll
        for (int q = 0; q < QN; q++) {
          const int c = cb + lane + 32 * q;
          uv[q] = c < nr ? us[k * nr + c] : R(0);
        }
#pragma unroll
        for (int t = 0; t < TR; t++)
#pragma unroll
          for (int q = 0; q < QN; q++) acc[t][q] = fma(-lr[t][k], uv[q], acc[t][q]);
      }
#pragma unroll
      for (int t = 0; t < TR; t++)
#pragma unroll
        for (int q = 0; q < QN; q++) {
          const int c = cb + lane + 32 * q;
          if (crow[t] && c < nr) crow[t][c] = P::cv(acc[t][q]);
        }
    }
  }
}

// Blocked right-looking LU with partial pivoting of M (n x n, pitch p, rows
// addressed through rmap: logical row i is physical row rmap[i]). On return
// rmap[i] = the original row now at position i (the reference's piv).
//   panel : columns [j0, j1) of logical rows >= j0 staged in st (pitch SP).
//           Staged rows never move: perm[r] is the staged row at logical
//           position j0 + r and spos[s] the logical position (relative to j0)
//           of staged row s. Thread t owns staged rows t, t + BT, ... Per
//           column jj: pivot search over own rows still at positions >= jj
//           (the reference's first-maximum rule, ties to the lowest logical
//           position, lu.rs:132-137), one barrier, then every thread picks the
//           winner from the warps' candidates, reads the pivot row in place,
//           and scales and updates its own rows; the row that was at position
//           jj takes the winner's position. Only thread 0 touches perm and
//           rmap, and the pivot row is never written after it is chosen, so
//           one barrier per column suffices (the candidate slots are
//           double-buffered by column parity).
//   U12   : rows [j0, j1), columns >= j1, each column solved in registers.
//   A22  -= L21 U12 (trailing_update).
// Values written back to M are rounded to the storage type, and the staged
// copies used by later steps are those rounded values.
template <typename P>
__device__ void block_lu(typename P::S* M, int p, int n, int* rmap, typename P::R* st,
                         typename P::R* us, Shared& sh) {
  const int BT = blockDim.x, NW = BT >> 5;
  using S = typename P::S;
  using R = typename P::R;
  constexpr int TR = 2;  // rows per thread in the A22 tile
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int* perm = rmap + n;
  int* spos = rmap + 2 * n;
  for (int i = tid; i < n; i += BT) rmap[i] = i;
  __syncthreads();
  for (int j0 = 0; j0 < n; j0 += PBW) {
    const int jb = min(PBW, n - j0), j1 = j0 + jb, prow = n - j0;
    for (int idx = tid; idx < prow * jb; idx += BT) {
      const int r = idx / jb, c = idx - r * jb;
      st[r * SP + c] = P::ld(&M[(size_t)rmap[j0 + r] * p + j0 + c]);
    }
    for (int r = tid; r < prow; r += BT) {
      perm[r] = r;
      spos[r] = r;
    }
    __syncthreads();
    for (int jj = 0; jj < jb; jj++) {
      const int par = jj & 1;
      unsigned long long bk = 0ull;
      int bp = -1, bs = -1;
      for (int s = tid; s < prow; s += BT) {
        const int ps = spos[s];
        if (ps >= jj) {
          const unsigned long long k = bkey<R>(st[s * SP + jj], ps, jj);
          if (bbetter(k, ps, bk, bp)) { bk = k; bp = ps; bs = s; }
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long ok = __shfl_down_sync(0xffffffffu, bk, off);
        const int op = __shfl_down_sync(0xffffffffu, bp, off);
        const int os = __shfl_down_sync(0xffffffffu, bs, off);
        if (bbetter(ok, op, bk, bp)) { bk = ok; bp = op; bs = os; }
      }
      if (lane == 0) { sh.rk[par][warp] = bk; sh.rp[par][warp] = bp; sh.rs[par][warp] = bs; }
      __syncthreads();
      bk = sh.rk[par][0];
      bp = sh.rp[par][0];
      bs = sh.rs[par][0];
      for (int w = 1; w < NW; w++)
        if (bbetter(sh.rk[par][w], sh.rp[par][w], bk, bp)) {
          bk = sh.rk[par][w]; bp = sh.rp[par][w]; bs = sh.rs[par][w];
        }
      // bp >= jj: the row at position jj always has a key.
      const R* prow_v = st + bs * SP;
      const R d = prow_v[jj];
      const R sc = d != R(0) ? R(1) / d : R(1);
      for (int s = tid; s < prow; s += BT) {
        int ps = spos[s];
        if (s == bs) {
          spos[s] = jj;
          continue;
        }
        if (ps == jj) {  // the row displaced from position jj goes to bp
          ps = bp;
          spos[s] = bp;
        }
        if (ps > jj) {
          R* row = st + s * SP;
          const R l = d != R(0) ? row[jj] * sc : row[jj];
          row[jj] = l;
          for (int c = jj + 1; c < jb; c++) row[c] = fma(-l, prow_v[c], row[c]);
        }
      }
      if (tid == 0 && bp != jj) {
        const int t = perm[jj];
        perm[jj] = perm[bp];
        perm[bp] = t;
        const int u = rmap[j0 + jj];
        rmap[j0 + jj] = rmap[j0 + bp];
        rmap[j0 + bp] = u;
      }
    }
    __syncthreads();
    for (int idx = tid; idx < prow * jb; idx += BT) {
      const int r = idx / jb, c = idx - r * jb;
      R* sv = st + perm[r] * SP + c;
      const S v = P::cv(*sv);
      M[(size_t)rmap[j0 + r] * p + j0 + c] = v;
      *sv = P::up(v);
    }
    if (j1 >= n) break;  // uniform; jb == PBW below
    const int nr = n - j1;
    for (int idx = tid; idx < PBW * nr; idx += BT) {
      const int k = idx / nr, c = idx - k * nr;
      us[k * nr + c] = P::ld(&M[(size_t)rmap[j0 + k] * p + j1 + c]);
    }
    __syncthreads();
    {
      const R* l11[PBW];
#pragma unroll
      for (int i = 0; i < PBW; i++) l11[i] = st + perm[i] * SP;
      for (int c = tid; c < nr; c += BT) {
        R u[PBW];
#pragma unroll
        for (int k = 0; k < PBW; k++) u[k] = us[k * nr + c];
#pragma unroll
        for (int k = 0; k < PBW; k++)
#pragma unroll
          for (int i = k + 1; i < PBW; i++) u[i] = fma(-l11[i][k], u[k], u[i]);
#pragma unroll
        for (int k = 0; k < PBW; k++) {
          const S v = P::cv(u[k]);
          M[(size_t)rmap[j0 + k] * p + j1 + c] = v;
          us[k * nr + c] = P::up(v);
        }
      }
    }
    __syncthreads();
    switch (min(4, (nr + 31) / 32)) {
      case 1: trailing_update<P, TR, 1>(M, p, rmap, j1, nr, st, us, perm); break;
      case 2: trailing_update<P, TR, 2>(M, p, rmap, j1, nr, st, us, perm); break;
      case 3: trailing_update<P, TR, 3>(M, p, rmap, j1, nr, st, us, perm); break;
      default: trailing_update<P, TR, 4>(M, p, rmap, j1, nr, st, us, perm); break;
    }
    __syncthreads();
  }
  __syncthreads();
}

// One row of a block step of the triangular solves: x_i -= f * X_blk over all
// nrhs right-hand sides, with the row's kbn (<= 16) factor entries f loaded
// once (16 independent loads in flight) and the block's solved values X_blk
// read from shared memory (the same address across the warp: a broadcast).
template <typename P, typename TX>
__device__ __forceinline__ void solve_row_update(const typename P::S* frow, int kbn, TX* xi,
                                                 const TX* xblk, int nrhs) {
  TX f[16];
#pragma unroll
  for (int k = 0; k < 16; k++) f[k] = k < kbn ? (TX)P::ld(&frow[k]) : TX(0);
#pragma unroll
  for (int c = 0; c < 4; c++) {
    if (c < nrhs) {
      TX s = xi[c];
#pragma unroll
      for (int k = 0; k < 16; k++)
        if (k < kbn) s = fma(-f[k], xblk[k * nrhs + c], s);
      xi[c] = s;
    }
  }
}

// X (n x nrhs, pitch nrhs, already in the factor's row order, i.e. P b)
// <- U^-1 L^-1 X with the stored factors in M. 16-row blocks: warp 0 solves
// the diagonal block (lanes = rows, two right-hand sides per pass, values
// passed by shuffles), then all threads update the remaining rows.
template <typename P, typename TX>
__device__ void block_solve(const typename P::S* M, int p, int n, const int* rmap, TX* X,
                            int nrhs) {
  const int BT = blockDim.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int li = lane & 15, half = lane >> 4;
  for (int kb = 0; kb < n; kb += 16) {
    const int kbn = min(16, n - kb);
    if (warp == 0) {
      // lane's row of the diagonal block in registers (16 loads in flight)
      const typename P::S* lrow = M + (size_t)rmap[kb + min(li, kbn - 1)] * p + kb;
      TX lv[16];
#pragma unroll
      for (int k = 0; k < 16; k++) lv[k] = k < kbn ? (TX)P::ld(&lrow[k]) : TX(0);
      for (int c0 = 0; c0 < nrhs; c0 += 2) {
        const int c = c0 + half;
        const bool act = li < kbn && c < nrhs;
        TX xi = act ? X[(kb + li) * nrhs + c] : TX(0);
#pragma unroll
        for (int k = 0; k < 15; k++) {
          if (k + 1 < kbn) {
            const TX xk = __shfl_sync(0xffffffffu, xi, (lane & 16) | k);
            if (act && li > k) xi = fma(-lv[k], xk, xi);
          }
        }
        if (act) X[(kb + li) * nrhs + c] = xi;
      }
    }
    __syncthreads();
    const int rest = n - kb - kbn;
    for (int r = tid; r < rest; r += BT)
      solve_row_update<P, TX>(M + (size_t)rmap[kb + kbn + r] * p + kb, kbn,
                              X + (size_t)(kb + kbn + r) * nrhs, X + (size_t)kb * nrhs, nrhs);
    __syncthreads();
  }
  for (int kb = (n - 1) / 16 * 16; kb >= 0; kb -= 16) {
    const int kbn = min(16, n - kb);
    if (warp == 0) {
      const typename P::S* urow = M + (size_t)rmap[kb + min(li, kbn - 1)] * p + kb;
      TX uv[16];
#pragma unroll
      for (int k = 0; k < 16; k++) uv[k] = k < kbn ? (TX)P::ld(&urow[k]) : TX(1);
      for (int c0 = 0; c0 < nrhs; c0 += 2) {
        const int c = c0 + half;
        const bool act = li < kbn && c < nrhs;
        TX xi = act ? X[(kb + li) * nrhs + c] : TX(0);
#pragma unroll
        for (int k = 15; k >= 0; k--) {
          if (k < kbn) {
            if (act && li == k) xi = xi / uv[k];
            const TX xk = __shfl_sync(0xffffffffu, xi, (lane & 16) | k);
            if (act && li < k) xi = fma(-uv[k], xk, xi);
          }
        }
        if (act) X[(kb + li) * nrhs + c] = xi;
      }
    }
    __syncthreads();
    for (int r = tid; r < kb; r += BT)
      solve_row_update<P, TX>(M + (size_t)rmap[r] * p + kb, kbn, X + (size_t)r * nrhs,
                              X + (size_t)kb * nrhs, nrhs);
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
  int* redo;         // [0] = count, [1 + k] = k-th system (sorted index) left for the FP64 pass
  int* status;       // per system (sorted order): iterations, < 0 = not converged
  double* eta;       // per system: final backward error (mixed pass) or -1
  void* scratch;     // per-CTA global working matrices for systems that do not fit
  size_t scratch_bytes;  // bytes per CTA slice
  size_t smem_budget;    // dynamic shared memory of each CTA
  int max_iters;
  double tol;
  int only_flagged;  // FP64 pass: process only systems with status < 0
  int gmres_m;       // largest Krylov basis of the GMRES-IR stage (0: no GMRES-IR)
  int* piv;          // per system at desc.poff: the row order (lu.rs piv) of the factors used
  long long* cycles; // per system: SM cycles spent on it, summed over the passes
  unsigned long long* phase;  // [8]: load, factor, solves, residuals of the first pass,
                              // then the same for the FP64 redo pass (summed over CTAs)
};

// Per-CTA phase clock: thread 0 adds the cycles since the last mark to a slot.
struct PhaseClock {
  long long last;
  unsigned long long acc[4];
  __device__ void start() {
    last = clock64();
    acc[0] = acc[1] = acc[2] = acc[3] = 0ull;
  }
  __device__ void mark(int k) {
    const long long t = clock64();
    acc[k] += (unsigned long long)(t - last);
    last = t;
  }
  __device__ void flush(unsigned long long* out) {
    for (int k = 0; k < 4; k++) atomicAdd(&out[k], acc[k]);
  }
};

// atomicMax on a non-negative double held in shared memory.
__device__ __forceinline__ void amax_pos(double* p, double v) {
  atomicMax(reinterpret_cast<unsigned long long*>(p), (unsigned long long)__double_as_longlong(v));
}

// out[c] = max over the CTA of |v[i nrhs + c]| (c < nrhs, n rows): per-thread
// maxima, then a warp reduction, then one shared atomic per warp and column.
// The maxima are taken on the magnitudes' bit patterns with integer
// instructions (they order like the values, and a NaN orders above every
// number, so a NaN residual can never pass the convergence test); the FP64
// pipe stays free for the residual. out must be zero on entry; no barrier
// inside.
__device__ __forceinline__ void col_absmax(const double* v, int n, int nrhs, double* out) {
  const int BT = blockDim.x;
  unsigned long long m[4] = {0ull, 0ull, 0ull, 0ull};
  for (int idx = threadIdx.x; idx < n * nrhs; idx += BT) {
    const int c = idx % nrhs;
    const unsigned long long a = la_absbits_f64(v[idx]);
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (q == c) m[q] = a > m[q] ? a : m[q];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, m[q], off);
      m[q] = o > m[q] ? o : m[q];
    }
    if ((threadIdx.x & 31) == 0 && q < nrhs)
      atomicMax(reinterpret_cast<unsigned long long*>(&out[q]), m[q]);
  }
}

// One halving step of a warp reduction of 2H values per lane: lanes with
// bit s set keep the upper H values, the others the lower H, each adding its
// partner's copy (partner = lane ^ s).
template <int H>
__device__ __forceinline__ void halve(double* v, int lane, int s) {
  const bool up = lane & s;
#pragma unroll
  for (int j = 0; j < H; j++) {
    const double send = up ? v[j] : v[j + H];
    const double keep = up ? v[j + H] : v[j];
    v[j] = keep + __shfl_xor_sync(0xffffffffu, send, s);
  }
}

// R = B - A x (or R = A x when MV) in FP64 for rows [0, n) with NR right-hand
// sides: each warp takes four rows at a time, lanes stride the columns
// (coalesced rows of A, x from shared memory), and the V = 4 CW partial sums
// (CW = NR rounded up to a power of two) are reduced across the warp by
// recursive halving, V - 1 adds per lane, followed by 5 - log2 V butterfly
// adds: 6, 9 and 16 FP64 adds per lane for 1, 2 and 4 right-hand sides.
template <int NR, bool MV = false>
__device__ void residual_rows(const double* __restrict__ Ai, int n, const double* xv,
                              const double* __restrict__ Bi, double* Ri) {
  constexpr int CW = NR == 1 ? 1 : (NR == 2 ? 2 : 4);
  constexpr int V = 4 * CW;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, NW = blockDim.x >> 5;
  for (int r0 = 4 * warp; r0 < n; r0 += 4 * NW) {
    double v[V];
#pragma unroll
    for (int j = 0; j < V; j++) v[j] = 0.0;
#pragma unroll 2
    for (int k0 = 0; k0 < n; k0 += 32) {
      const int k = k0 + lane;
      const bool kin = k < n;
      double a[4], xk[NR];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = (kin && r0 + i < n) ? Ai[(size_t)(r0 + i) * n + k] : 0.0;
#pragma unroll
      for (int c = 0; c < NR; c++) xk[c] = kin ? xv[k * NR + c] : 0.0;
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int c = 0; c < NR; c++) v[i * CW + c] = fma(a[i], xk[c], v[i * CW + c]);
    }
    // Halving: after the step with lane bit s, a lane keeps the half of its
    // values selected by that bit. The value index q = i CW + c ends up with
    // its top bit chosen by lane bit 16, the next by lane bit 8, and so on.
    if constexpr (V == 16) halve<8>(v, lane, 16);
    if constexpr (V >= 8) halve<4>(v, lane, V == 16 ? 8 : 16);
    halve<2>(v, lane, V == 16 ? 4 : (V == 8 ? 8 : 16));
    halve<1>(v, lane, V == 16 ? 2 : (V == 8 ? 4 : 8));
    // Butterfly over the lane bits below the ones used for halving.
    constexpr int LB = V == 16 ? 4 : (V == 8 ? 3 : 2);  // lane bits used by halving
#pragma unroll
    for (int s = (16 >> LB); s >= 1; s >>= 1) v[0] += __shfl_xor_sync(0xffffffffu, v[0], s);
    // q's bits (most significant first) are lane bits 16, 8, ... (LB of them).
    int q = 0;
#pragma unroll
    for (int t = 0; t < LB; t++) q = q * 2 + ((lane >> (4 - t)) & 1);
    const int i = q / CW, c = q % CW;
    const bool leader = (lane & ((32 >> LB) - 1)) == 0;
    if (leader && c < NR && r0 + i < n)
      Ri[(size_t)(r0 + i) * NR + c] = MV ? v[0] : Bi[(size_t)(r0 + i) * NR + c] - v[0];
  }
}

__device__ __forceinline__ double block_sum_d(double s, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, NW = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) red[warp] = s;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < NW; w++) t += red[w];
  __syncthreads();
  return t;
}

__device__ __forceinline__ double block_max_d(double s, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, NW = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
  if (lane == 0) red[warp] = s;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < NW; w++) t = fmax(t, red[w]);
  __syncthreads();
  return t;
}

// Normwise backward error max_c ||r_c||_inf / (||A||_inf ||x_c||_inf + ||b_c||_inf)
// of the current (x, r); leaves max |r_c| in sh.norm[1 + c].
__device__ double refine_eta(const double* rv, const double* xv, int n, int nrhs, Shared& sh) {
  if (threadIdx.x < 8) sh.norm[1 + threadIdx.x] = 0.0;
  __syncthreads();
  col_absmax(rv, n, nrhs, &sh.norm[1]);
  col_absmax(xv, n, nrhs, &sh.norm[1 + 4]);
  __syncthreads();
  double eta = 0.0;
  for (int c = 0; c < nrhs; c++) {
    const double den = sh.norm[0] * sh.norm[1 + 4 + c] + sh.norm[1 + 8 + c];
    const double v = den > 0 ? sh.norm[1 + c] / den : (sh.norm[1 + c] > 0 ? INFINITY : 0.0);
    if (!(v <= eta)) eta = v;
  }
  return eta;
}

// w <- A^-1 w through the stored factors of scale * A: an FP32 solve of
// P w / max|w| (the preconditioner of GMRES-IR).
template <typename P>
__device__ void precondition(const typename P::S* M, int n, const int* rmap, double* w, float* dv,
                             float scale, Shared& sh) {
  const int BT = blockDim.x;
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += BT) m = fmax(m, fabs(w[i]));
  m = block_max_d(m, sh.red);
  const double inv = m > 0 ? 1.0 / m : 0.0;
  for (int i = threadIdx.x; i < n; i += BT) dv[i] = (float)(w[rmap[i]] * inv);
  __syncthreads();
  block_solve<P, float>(M, n, n, rmap, dv, 1);
  for (int i = threadIdx.x; i < n; i += BT) w[i] = (double)dv[i] * m * (double)scale;
  __syncthreads();
}

// One GMRES-IR correction of column c: solves (LU)^-1 A d = (LU)^-1 r_c by
// GMRES (FP64 Arnoldi with modified Gram-Schmidt and Givens rotations,
// basis V in global scratch, at most mcap steps, stopping when the estimated
// preconditioned residual falls below GM_TOL times its start), then x_c += d.
// Returns the steps taken.
template <typename P>
__device__ int gmres_column(const double* __restrict__ Ai, int n, int nrhs, int c,
                            const typename P::S* M, const int* rmap, const double* rv, double* xv,
                            float* dv, float scale, double* w, double* H, double* V, int mcap,
                            Shared& sh) {
  const int tid = threadIdx.x, BT = blockDim.x;
  double* g = H + (GM_M + 1) * GM_M;
  double* cs = g + GM_M + 1;
  double* sn = cs + GM_M + 1;
  for (int i = tid; i < n; i += BT) w[i] = rv[(size_t)i * nrhs + c];
  __syncthreads();
  precondition<P>(M, n, rmap, w, dv, scale, sh);
  double s = 0.0;
  for (int i = tid; i < n; i += BT) s += w[i] * w[i];
  const double beta = sqrt(block_sum_d(s, sh.red));
  if (!(beta > 0.0) || !(beta < INFINITY)) return 0;
  for (int i = tid; i < n; i += BT) V[i] = w[i] / beta;
  if (tid == 0) g[0] = beta;
  __syncthreads();
  int k = 0;
  for (int j = 0; j < mcap; j++) {
    residual_rows<1, true>(Ai, n, V + (size_t)j * n, nullptr, w);  // w = A v_j
    __syncthreads();
    precondition<P>(M, n, rmap, w, dv, scale, sh);
    for (int i = 0; i <= j; i++) {
      const double* vi = V + (size_t)i * n;
      double hs = 0.0;
      for (int t = tid; t < n; t += BT) hs += vi[t] * w[t];
      const double h = block_sum_d(hs, sh.red);
      for (int t = tid; t < n; t += BT) w[t] -= h * vi[t];
      if (tid == 0) H[i * GM_M + j] = h;
    }
    double hs = 0.0;
    for (int t = tid; t < n; t += BT) hs += w[t] * w[t];
    const double hn = sqrt(block_sum_d(hs, sh.red));
    double* vn = V + (size_t)(j + 1) * n;
    for (int t = tid; t < n; t += BT) vn[t] = hn > 0 ? w[t] / hn : 0.0;
    if (tid == 0) {
      for (int i = 0; i < j; i++) {
        const double h0 = H[i * GM_M + j], h1 = H[(i + 1) * GM_M + j];
        H[i * GM_M + j] = cs[i] * h0 + sn[i] * h1;
        H[(i + 1) * GM_M + j] = -sn[i] * h0 + cs[i] * h1;
      }
      const double h0 = H[j * GM_M + j];
      const double r = hypot(h0, hn);
      const double cj = r > 0 ? h0 / r : 1.0, sj = r > 0 ? hn / r : 0.0;
      cs[j] = cj;
      sn[j] = sj;
      H[j * GM_M + j] = r;
      g[j + 1] = -sj * g[j];
      g[j] = cj * g[j];
      sh.gres = fabs(g[j + 1]);
    }
    __syncthreads();
    k = j + 1;
    if (!(sh.gres > GM_TOL * beta) || !(hn > 0)) break;
  }
  if (tid == 0) {  // H(0:k, 0:k) y = g, y over g
    for (int i = k - 1; i >= 0; i--) {
      double t = g[i];
      for (int l = i + 1; l < k; l++) t -= H[i * GM_M + l] * g[l];
      g[i] = H[i * GM_M + i] != 0.0 ? t / H[i * GM_M + i] : 0.0;
    }
  }
  __syncthreads();
  for (int t = tid; t < n; t += BT) {
    double d = 0.0;
    for (int i = 0; i < k; i++) d += g[i] * V[(size_t)i * n + t];
    xv[(size_t)t * nrhs + c] += d;
  }
  __syncthreads();
  return k;
}

__device__ __forceinline__ void residual_all(const double* Ai, int n, int nrhs, const double* xv,
                                             const double* Bi, double* Ri) {
  switch (nrhs) {
    case 1: residual_rows<1>(Ai, n, xv, Bi, Ri); break;
    case 2: residual_rows<2>(Ai, n, xv, Bi, Ri); break;
    case 3: residual_rows<3>(Ai, n, xv, Bi, Ri); break;
    default: residual_rows<4>(Ai, n, xv, Bi, Ri); break;
  }
}

// One system on the whole CTA: factor in storage P, then (mixed) refine.
template <typename P, bool MIXED>
__device__ void process_system(const BatchArgs& a, int sidx, const SysDesc& d, Shared& sh,
                               char* smem) {
  const int BT = blockDim.x, NW = BT >> 5;
  using S = typename P::S;
  using R = typename P::R;
  const int tid = threadIdx.x;
  const int n = d.n, nrhs = d.nrhs;
  const Lay Lres = lay<S, R>(n, nrhs, true, MIXED);
  const bool resident = Lres.total <= a.smem_budget;
  const Lay L = resident ? Lres : lay<S, R>(n, nrhs, false, MIXED);
  S* M = resident ? reinterpret_cast<S*>(smem)
                  : reinterpret_cast<S*>(static_cast<char*>(a.scratch) +
                                         (size_t)blockIdx.x * a.scratch_bytes);
  R* st = reinterpret_cast<R*>(smem + L.stage);
  R* us = reinterpret_cast<R*>(smem + L.us);
  int* rmap = reinterpret_cast<int*>(smem + L.rmap);
  double* xv = reinterpret_cast<double*>(smem + L.x);
  float* dv = reinterpret_cast<float*>(smem + L.d);
  const double* Ai = a.A + d.a;
  const double* Bi = a.B + d.b;
  double* Xi = a.X + d.b;
  PhaseClock pc;
  if (tid == 0) pc.start();
  unsigned long long* const phase = a.phase + (a.only_flagged ? 4 : 0);

  // Storage scale (a power of two): the largest finite |a_ij| goes to 16 for
  // FP8, so the factors (|l| <= 1, modest growth in U) stay inside e4m3's
  // range. The maximum is taken on the magnitudes' bit patterns (integer
  // instructions: the FP64 pipe is GB300's scarcest unit).
  if (tid == 0) { sh.norm[0] = 0.0; sh.norm[13] = 0.0; }
  __syncthreads();
  float scale = 1.f;
  if (sizeof(S) == 1) {
    unsigned long long m = 0ull;
    for (int idx = tid; idx < n * n; idx += BT) {
      const unsigned long long a = la_absbits_f64(Ai[idx]);
      if (a < 0x7ff0000000000000ull && a > m) m = a;
    }
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long o = __shfl_down_sync(0xffffffffu, m, off);
      m = o > m ? o : m;
    }
    if ((tid & 31) == 0) atomicMax(reinterpret_cast<unsigned long long*>(&sh.norm[13]), m);
    __syncthreads();
    const unsigned long long mb = reinterpret_cast<const unsigned long long&>(sh.norm[13]);
    if (mb > 0ull) {
      // 2^(4 - e) with mb = 0.f * 2^e (0.5 <= f < 1), from the biased
      // exponent; subnormal maxima (e <= -1022) clamp to the FP32 range.
      const int e = (int)(mb >> 52) - 1022;
      scale = ldexpf(1.f, max(-126, min(127, 4 - e)));
    }
  }
  // Load A_i (one warp per row, coalesced) in the storage type. The low
  // precisions convert with integer instructions (la_f64_to_f32), and the
  // mixed pass takes ||A||_inf (largest row sum of |a_ij|) in FP32 on the way:
  // each row sum is a lower bound of the exact one after the factor
  // (1 - 2^-19), which covers the conversion and FP32 summation errors, so the
  // backward error computed with it never understates the exact one.
  {
    const int lane = tid & 31, warp = tid >> 5;
    float rmax = 0.f;
    for (int r = warp; r < n; r += NW) {
      const double* ar = Ai + (size_t)r * n;
      S* mr = M + (size_t)r * n;
      float rs = 0.f;
      // Eight loads per lane are issued before any conversion or store.
      for (int k0 = 0; k0 < n; k0 += 256) {
        double v8[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int k = k0 + lane + 32 * q;
          v8[q] = k < n ? __ldg(ar + k) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const int k = k0 + lane + 32 * q;
          if (k < n) {
            if constexpr (sizeof(S) == 8) {
              mr[k] = v8[q];
            } else {
              float v = la_f64_to_f32(v8[q]);
              if (MIXED) rs += fabsf(v);
              if (sizeof(S) == 1) v *= scale;
              mr[k] = P::cv(v);
            }
          }
        }
      }
      if (MIXED) {
        for (int off = 16; off > 0; off >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, off);
        rmax = fmaxf(rmax, rs);
      }
    }
    if (MIXED && lane == 0)
      amax_pos(&sh.norm[0], la_f32_to_f64(rmax) * (1.0 - 0x1p-19));
  }
  __syncthreads();
  if (tid == 0) pc.mark(0);
  block_lu<P>(M, n, n, rmap, st, us, sh);
  if (tid == 0) pc.mark(1);
  for (int i = tid; i < n; i += BT) a.piv[d.poff + i] = rmap[i];

  if (!MIXED) {
    for (int idx = tid; idx < n * nrhs; idx += BT) {
      const int i = idx / nrhs, c = idx - i * nrhs;
      xv[idx] = Bi[(size_t)rmap[i] * nrhs + c];
    }
    __syncthreads();
    block_solve<P, double>(M, n, n, rmap, xv, nrhs);
    for (int idx = tid; idx < n * nrhs; idx += BT) Xi[idx] = xv[idx];
    if (tid == 0) {
      a.status[sidx] = 0;
      a.eta[sidx] = -1.0;
      pc.mark(2);
      if (a.phase) pc.flush(phase);
    }
    return;
  }
  // ---- FP64 refinement with the stored factors (of scale * A) ----
  // The residual r = B - A x lives in X_i (global) until the final x is written.
  if (tid == 0) for (int q = 1; q < 13; q++) sh.norm[q] = 0.0;
  __syncthreads();
  col_absmax(Bi, n, nrhs, &sh.norm[1 + 2 * 4]);
  for (int idx = tid; idx < n * nrhs; idx += BT) xv[idx] = 0.0;
  __syncthreads();
  const double* rv = Bi;  // x = 0: r = B
  int it = 0;
  double eta = INFINITY, prev = INFINITY;
  bool ok = false;
  // LU-IR: x += LU \ r while the backward error drops by 10% per step.
  for (;;) {
    eta = refine_eta(rv, xv, n, nrhs, sh);
    if (eta <= a.tol) { ok = true; break; }
    if (it >= a.max_iters || !(eta < 0.9 * prev)) break;
    prev = eta;
    it++;
    // d = P r / rmax (the factor's row order)
    {
      double inv[4];
#pragma unroll
      for (int c = 0; c < 4; c++) inv[c] = sh.norm[1 + c] > 0 ? 1.0 / sh.norm[1 + c] : 0.0;
      for (int idx = tid; idx < n * nrhs; idx += BT) {
        const int i = idx / nrhs, c = idx - i * nrhs;
        const double ic = c == 0 ? inv[0] : c == 1 ? inv[1] : c == 2 ? inv[2] : inv[3];
        dv[idx] = la_f64_to_f32(rv[(size_t)rmap[i] * nrhs + c] * ic);
      }
    }
    __syncthreads();
    if (tid == 0) pc.mark(3);
    block_solve<P, float>(M, n, n, rmap, dv, nrhs);
    if (tid == 0) pc.mark(2);
    // (scale A) d = r / rmax  =>  A (scale d rmax) = r
    for (int idx = tid; idx < n * nrhs; idx += BT)
      xv[idx] = fma(la_f32_to_f64(dv[idx]), sh.norm[1 + idx % nrhs] * (double)scale, xv[idx]);
    __syncthreads();
    residual_all(Ai, n, nrhs, xv, Bi, Xi);
    rv = Xi;
    __syncthreads();
  }
  // GMRES-IR when LU-IR made progress (its best backward error went below
  // GM_TRIGGER) and then stalled: the same factors precondition GMRES in FP64,
  // as long as its matrix-vector products (steps x nrhs x n^2) stay below
  // half of what the FP64 redo would cost (n^3 / 3). Systems on which LU-IR
  // diverged from the start (kappa u_factor >> 1) go straight to the FP64 pass.
  int gsteps = 0;
  const int mcap = min(a.gmres_m, n / (2 * nrhs));
  if (!ok && mcap >= 4 && fmin(eta, prev) < GM_TRIGGER) {
    double* w = reinterpret_cast<double*>(smem + L.gm);
    double* H = w + n;
    double* V = reinterpret_cast<double*>(static_cast<char*>(a.scratch) +
                                          (size_t)blockIdx.x * a.scratch_bytes + GM_V_OFFSET);
    for (int outer = 0; outer < GM_OUTER && !ok; outer++) {
      for (int c = 0; c < nrhs; c++)
        gsteps += gmres_column<P>(Ai, n, nrhs, c, M, rmap, rv, xv, dv, scale, w, H, V, mcap, sh);
      residual_all(Ai, n, nrhs, xv, Bi, Xi);
      rv = Xi;
      __syncthreads();
      eta = refine_eta(rv, xv, n, nrhs, sh);
      if (eta <= a.tol) ok = true;
    }
  }
  __syncthreads();
  for (int idx = tid; idx < n * nrhs; idx += BT) Xi[idx] = xv[idx];
  if (tid == 0) {
    a.status[sidx] = ok ? it + gsteps : -1 - (it + gsteps);
    if (!ok) a.redo[1 + atomicAdd(&a.redo[0], 1)] = sidx;
    a.eta[sidx] = eta;
    pc.mark(3);
    if (a.phase) pc.flush(phase);
  }
}

// Storage classes of the mixed pass; CLS_F64 systems skip it and go straight
// to the FP64 pass.
enum { CLS_F64 = 0, CLS_F32 = 1, CLS_BF16 = 2, CLS_FP8 = 3 };

template <bool MIXED>
__global__ void __launch_bounds__(BT_MAX, MIXED ? 2 : 1) batched_kernel(BatchArgs a) {
  extern __shared__ __align__(16) double bsm[];
  __shared__ Shared sh;
  __shared__ int s_sys;
  const int tid = threadIdx.x;
  // The FP64 pass of a mixed plan works through the list of systems the mixed
  // pass could not refine, instead of visiting every system.
  for (;;) {
    if (tid == 0) {
      const int q = atomicAdd(a.queue, 1);
      const int total = a.only_flagged ? a.redo[0] : a.count;
      s_sys = q < total ? (a.only_flagged ? a.redo[1 + q] : q) : -1;
    }
    __syncthreads();
    const int sidx = s_sys;
    __syncthreads();
    if (sidx < 0) return;
    const SysDesc d = a.desc[sidx];
    char* smem = reinterpret_cast<char*>(bsm);
    const long long t0 = clock64();
    if (!MIXED) {
      process_system<StF64, false>(a, sidx, d, sh, smem);
    } else if (d.cls == CLS_F64) {
      if (tid == 0) {
        a.status[sidx] = -1;
        a.eta[sidx] = INFINITY;
        a.redo[1 + atomicAdd(&a.redo[0], 1)] = sidx;
      }
    } else if (d.cls == CLS_FP8) {
      process_system<StFP8, true>(a, sidx, d, sh, smem);
    } else if (d.cls == CLS_BF16) {
      process_system<StBF16, true>(a, sidx, d, sh, smem);
    } else {
      process_system<StF32, true>(a, sidx, d, sh, smem);
    }
    __syncthreads();
    if (tid == 0) a.cycles[sidx] += clock64() - t0;
  }
}

// desc[i].cls from the selector's class (0 FP8, 1 BF16, 2 FP32, 3 straight to
// the FP64 pass) of the caller's system perm[i].
__global__ void select_kernel(SysDesc* desc, const int* __restrict__ perm,
                              const int* __restrict__ sel, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int c = sel[perm[i]];
  desc[i].cls = c == 0 ? CLS_FP8 : (c == 1 ? CLS_BF16 : (c == 3 ? CLS_F64 : CLS_F32));
}

constexpr size_t BATCH_STATIC_SMEM = 1024;  // bound of the kernel's static shared memory

}  // namespace

struct la_batch_plan_s {
  la_ctx ctx;
  int count = 0, mode = 0, ctas_per_sm = 1, threads = BT_MAX, gmres_m = 0;
  double tol = 1e-14;
  int max_iters = 10;
  const double *A = nullptr, *B = nullptr;
  double* X = nullptr;
  SysDesc* d_desc = nullptr;
  int* d_queue = nullptr;
  int* d_redo = nullptr;
  int* d_status = nullptr;
  double* d_eta = nullptr;
  long long* d_cycles = nullptr;
  unsigned long long* d_phase = nullptr;
  int* d_perm = nullptr;
  int* d_piv = nullptr;     // row orders, system after system in queue order
  std::vector<int> poff;    // caller's system -> offset in d_piv
  std::vector<int> n_of;    // caller's system -> n
  long long piv_total = 0;
  void* d_scratch = nullptr;
  std::vector<int> perm;  // sorted position -> caller's system index
  size_t smem = 0, smem_fp64 = 0, scratch_bytes = 0;
  int grid = 0, grid_fp64 = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

template <bool MIXED>
la_status set_kernel_smem(la_ctx ctx) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, batched_kernel<MIXED>);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaFuncGetAttributes(batched)");
  if (fa.sharedSizeBytes > BATCH_STATIC_SMEM) {
    ctx->last_error = "batched_kernel static shared memory exceeds its reserved bound";
    return LA_UNSUPPORTED;
  }
  e = cudaFuncSetAttribute(batched_kernel<MIXED>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(ctx->smem_optin - BATCH_STATIC_SMEM));
  return e == cudaSuccess ? LA_OK : la_cuda_fail(ctx, e, "cudaFuncSetAttribute(batched)");
}

// CTAs of batched_kernel<MIXED> that fit on one SM with `threads` threads and
// `smem` bytes of dynamic shared memory each.
template <bool MIXED>
int resident_ctas(int threads, size_t smem) {
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, batched_kernel<MIXED>, threads,
                                                    smem) != cudaSuccess)
    return 0;
  return blocks;
}

template <bool MIXED>
la_status launch_pass(la_batch_plan_s* pl, int* queue, int only_flagged, size_t smem, int grid,
                      int threads) {
  la_ctx ctx = pl->ctx;
  BatchArgs a;
  a.A = pl->A;
  a.B = pl->B;
  a.X = pl->X;
  a.desc = pl->d_desc;
  a.count = pl->count;
  a.queue = queue;
  a.redo = pl->d_redo;
  a.status = pl->d_status;
  a.eta = pl->d_eta;
  a.scratch = pl->d_scratch;
  a.scratch_bytes = pl->scratch_bytes;
  a.smem_budget = smem;
  a.max_iters = pl->max_iters;
  a.tol = pl->tol;
  a.only_flagged = only_flagged;
  a.gmres_m = pl->gmres_m;
  a.cycles = pl->d_cycles;
  a.piv = pl->d_piv;
  a.phase = pl->d_phase;
  batched_kernel<MIXED><<<grid, threads, smem, ctx->stream>>>(a);
  ctx->launches++;
  return la_check_launch(ctx, "batched_kernel");
}

// The whole pipeline on the context's stream.
la_status enqueue_plan(la_batch_plan_s* pl) {
  la_ctx ctx = pl->ctx;
  LA_CUDA(ctx, cudaMemsetAsync(pl->d_queue, 0, 2 * sizeof(int), ctx->stream));
  LA_CUDA(ctx, cudaMemsetAsync(pl->d_redo, 0, sizeof(int), ctx->stream));
  LA_CUDA(ctx, cudaMemsetAsync(pl->d_cycles, 0, pl->count * sizeof(long long), ctx->stream));
  LA_CUDA(ctx, cudaMemsetAsync(pl->d_phase, 0, 8 * sizeof(unsigned long long), ctx->stream));
  if (pl->mode == LA_BATCH_FP64) {
    LA_TRY(launch_pass<false>(pl, pl->d_queue, 0, pl->smem, pl->grid, pl->threads));
  } else {
    LA_TRY(launch_pass<true>(pl, pl->d_queue, 0, pl->smem, pl->grid, pl->threads));
    // FP64 pass over systems whose refinement did not converge: one
    // 256-thread CTA per SM with all of its shared memory.
    LA_TRY(launch_pass<false>(pl, pl->d_queue + 1, 1, pl->smem_fp64, pl->grid_fp64, BT_MAX));
  }
  return LA_OK;
}

int class_of(int prec) {
  switch (prec) {
    case LA_PREC_FP8: return CLS_FP8;
    case LA_PREC_BF16: return CLS_BF16;
    case LA_PREC_FP64: return CLS_F64;
    default: return CLS_F32;
  }
}

}  // namespace

extern "C" {

la_status la_batch_plan_create(la_ctx ctx, const double* d_a, const double* d_b, double* d_x,
                               const la_batch_system* systems, int count, int mode,
                               int ctas_per_sm, int warps_per_system, double tol, int max_iters,
                               la_batch_plan* out) {
  if (!ctx || !d_a || !d_b || !d_x || !systems || !out || count <= 0) return LA_INVALID;
  if (mode != LA_BATCH_FP64 && mode != LA_BATCH_MIXED) return LA_INVALID;
  if (warps_per_system == 0) warps_per_system = NW_MAX;
  if (ctas_per_sm < 1 || ctas_per_sm > 8) return LA_INVALID;
  if (warps_per_system != 2 && warps_per_system != 4 && warps_per_system != 8) return LA_INVALID;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  int nmax = 0;
  for (int i = 0; i < count; i++) {
    if (systems[i].n < 1 || systems[i].n > NMAX || systems[i].nrhs < 1 || systems[i].nrhs > 4)
      return LA_UNSUPPORTED;
    nmax = std::max(nmax, systems[i].n);
  }
  LA_TRY(set_kernel_smem<true>(ctx));
  LA_TRY(set_kernel_smem<false>(ctx));
  // Per-CTA budget: ctas_per_sm CTAs share an SM's shared memory. Every system
  // of the batch must fit with its matrix in global scratch; the FP64 redo
  // pass of a mixed plan has a whole SM per CTA.
  const size_t optin = (size_t)ctx->smem_optin - BATCH_STATIC_SMEM;
  const size_t budget =
      std::min(optin, (size_t)(228 * 1024) / ctas_per_sm - 1024 - BATCH_STATIC_SMEM);
  const int threads = 32 * warps_per_system;
  const size_t need = mode == LA_BATCH_FP64
                          ? lay<double, double>(nmax, 4, false, false).total
                          : lay<float, float>(nmax, 4, false, true).total;
  if (budget < need) return LA_UNSUPPORTED;
  if (lay<double, double>(NMAX, 4, false, false).total > optin) return LA_UNSUPPORTED;
  const int fit = mode == LA_BATCH_FP64 ? resident_ctas<false>(threads, budget)
                                        : resident_ctas<true>(threads, budget);
  if (fit < ctas_per_sm) return LA_UNSUPPORTED;
  la_batch_plan_s* pl = new (std::nothrow) la_batch_plan_s();
  if (!pl) return LA_NOMEM;
  pl->ctx = ctx;
  pl->count = count;
  pl->mode = mode;
  pl->ctas_per_sm = ctas_per_sm;
  pl->threads = threads;
  pl->gmres_m = mode == LA_BATCH_MIXED ? std::min(ctx->batch_gmres, GM_M) : 0;
  pl->tol = tol;
  pl->max_iters = max_iters;
  pl->A = d_a;
  pl->B = d_b;
  pl->X = d_x;
  pl->smem = budget;
  pl->smem_fp64 = optin;
  pl->grid = ctx->sm_count * ctas_per_sm;
  pl->grid_fp64 = ctx->sm_count;
  pl->scratch_bytes = al16((size_t)NMAX * NMAX * sizeof(double));
  // Work queue order: decreasing n (cost ~ n^3), ties by index.
  pl->perm.resize(count);
  for (int i = 0; i < count; i++) pl->perm[i] = i;
  std::stable_sort(pl->perm.begin(), pl->perm.end(),
                   [&](int x, int y) { return systems[x].n > systems[y].n; });
  std::vector<SysDesc> h(count);
  pl->poff.assign(count, 0);
  pl->n_of.resize(count);
  for (int i = 0; i < count; i++) pl->n_of[i] = systems[i].n;
  long long off = 0;
  for (int i = 0; i < count; i++) {
    const la_batch_system& s = systems[pl->perm[i]];
    h[i].a = (long long)s.a_offset;
    h[i].b = (long long)s.b_offset;
    h[i].n = s.n;
    h[i].nrhs = s.nrhs;
    h[i].cls = class_of(s.precision);
    h[i].poff = (int)off;
    pl->poff[pl->perm[i]] = (int)off;
    off += s.n;
  }
  pl->piv_total = off;  // at most count * 512, checked below
  const int slices = std::max(pl->grid, pl->grid_fp64);
  la_status s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_desc), count * sizeof(SysDesc));
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_queue), 64);
  if (s == LA_OK)
    s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_redo), (size_t)(count + 1) * sizeof(int));
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_status), count * sizeof(int));
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_eta), count * sizeof(double));
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_cycles), count * sizeof(long long));
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_perm), count * sizeof(int));
  if (s == LA_OK && pl->piv_total > INT32_MAX) s = LA_UNSUPPORTED;
  if (s == LA_OK)
    s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_piv), (size_t)pl->piv_total * sizeof(int));
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&pl->d_phase), 8 * sizeof(unsigned long long));
  if (s == LA_OK) s = la_device_alloc(ctx, &pl->d_scratch, (size_t)slices * pl->scratch_bytes);
  if (s == LA_OK) {
    cudaError_t e = cudaMemcpyAsync(pl->d_desc, h.data(), count * sizeof(SysDesc),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(pl->d_perm, pl->perm.data(), count * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(pl->d_status, 0, count * sizeof(int), ctx->stream);
    if (e != cudaSuccess) s = la_cuda_fail(ctx, e, "batch plan upload");
  }
  if (s == LA_OK) s = la_sync_and_check(ctx, "batch plan");
  // One uncaptured run, then the graph.
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
    if (iterations) iterations[orig] = st[i] >= 0 ? st[i] : -1 - st[i];
    if (eta) eta[orig] = et[i];
    // The FP64 pass leaves eta = -1 on the systems it redid.
    if (fell_back) fell_back[orig] = (pl->mode == LA_BATCH_MIXED && et[i] < 0.0) ? 1 : 0;
  }
  return LA_OK;
}

la_status la_batch_partition(const la_batch_system* systems, int count, int parts, int* bounds) {
  if (!systems || !bounds || count < 0 || parts < 1) return LA_INVALID;
  // cost of system i: its LU and solve flops, 2/3 n^3 + 2 n^2 nrhs
  std::vector<double> cum((size_t)count + 1, 0.0);
  for (int i = 0; i < count; i++) {
    const double n = systems[i].n, r = systems[i].nrhs;
    if (systems[i].n < 1 || systems[i].nrhs < 1) return LA_BADSHAPE;
    cum[i + 1] = cum[i] + 2.0 / 3.0 * n * n * n + 2.0 * n * n * r;
  }
  const double total = cum[count];
  bounds[0] = 0;
  int lo = 0;
  for (int p = 1; p < parts; p++) {
    // the boundary whose cumulative cost is nearest to p / parts of the total
    const double target = total * p / parts;
    int b = (int)(std::lower_bound(cum.begin() + lo, cum.end(), target) - cum.begin());
    if (b > lo && b <= count && target - cum[b - 1] < cum[b] - target) b--;
    b = std::min(std::max(b, lo), count);
    bounds[p] = b;
    lo = b;
  }
  bounds[parts] = count;
  return LA_OK;
}

la_status la_batch_plan_pivots(la_batch_plan pl, uint64_t* piv) {
  if (!pl || !piv) return LA_INVALID;
  la_ctx ctx = pl->ctx;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  std::vector<int> p((size_t)pl->piv_total);
  LA_CUDA(ctx, cudaMemcpyAsync(p.data(), pl->d_piv, p.size() * sizeof(int),
                               cudaMemcpyDeviceToHost, ctx->stream));
  LA_TRY(la_sync_and_check(ctx, "batch pivots"));
  // Device order is the work queue's; the caller's order packs the systems
  // one after the other as given.
  size_t out = 0;
  for (int i = 0; i < pl->count; i++) {
    const int n = pl->n_of[i];
    for (int r = 0; r < n; r++) piv[out + r] = (uint64_t)p[(size_t)pl->poff[i] + r];
    out += n;
  }
  return LA_OK;
}

la_status la_batch_plan_select_device(la_batch_plan pl, const int* d_class) {
  if (!pl || !d_class) return LA_INVALID;
  if (pl->mode != LA_BATCH_MIXED) return LA_INVALID;
  la_ctx ctx = pl->ctx;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  select_kernel<<<(pl->count + 255) / 256, 256, 0, ctx->stream>>>(pl->d_desc, pl->d_perm, d_class,
                                                                  pl->count);
  ctx->launches++;
  return la_check_launch(ctx, "select_kernel");
}

la_status la_batch_plan_phase_cycles(la_batch_plan pl, long long* phase) {
  if (!pl || !phase) return LA_INVALID;
  la_ctx ctx = pl->ctx;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  LA_CUDA(ctx, cudaMemcpyAsync(phase, pl->d_phase, 8 * sizeof(long long), cudaMemcpyDeviceToHost,
                               ctx->stream));
  return la_sync_and_check(ctx, "batch phase cycles");
}

la_status la_batch_plan_cycles(la_batch_plan pl, long long* cycles) {
  if (!pl || !cycles) return LA_INVALID;
  la_ctx ctx = pl->ctx;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  std::vector<long long> c(pl->count);
  LA_CUDA(ctx, cudaMemcpyAsync(c.data(), pl->d_cycles, pl->count * sizeof(long long),
                               cudaMemcpyDeviceToHost, ctx->stream));
  LA_TRY(la_sync_and_check(ctx, "batch cycles"));
  for (int i = 0; i < pl->count; i++) cycles[pl->perm[i]] = c[i];
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
  la_device_free(ctx, pl->d_redo);
  la_device_free(ctx, pl->d_status);
  la_device_free(ctx, pl->d_eta);
  la_device_free(ctx, pl->d_cycles);
  la_device_free(ctx, pl->d_perm);
  la_device_free(ctx, pl->d_piv);
  la_device_free(ctx, pl->d_phase);
  la_device_free(ctx, pl->d_scratch);
  cudaStreamSynchronize(ctx->stream);
  delete pl;
}

la_status la_batch_autotune(la_ctx ctx, const double* d_a, const double* d_b, double* d_x,
                            const la_batch_system* systems, int count, int mode, double tol,
                            int max_iters, const char* table_path, int* best_ctas_per_sm,
                            int* best_warps_per_system, double* best_ms) {
  if (!ctx || !best_ctas_per_sm || !systems || count <= 0) return LA_INVALID;
  double mean_n = 0;
  for (int i = 0; i < count; i++) mean_n += systems[i].n;
  mean_n /= count;
  int best_c = 0, best_w = 0;
  double best_t = INFINITY;
  struct Row { int c, w; double ms; };
  std::vector<Row> rows;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  LA_CUDA(ctx, cudaEventCreate(&e0));
  LA_CUDA(ctx, cudaEventCreate(&e1));
  const int warps[3] = {8, 4, 2};
  const int ctas[4] = {1, 2, 4, 8};
  for (int w : warps)
    for (int c : ctas) {
      la_batch_plan pl = nullptr;
      if (la_batch_plan_create(ctx, d_a, d_b, d_x, systems, count, mode, c, w, tol, max_iters,
                               &pl) != LA_OK)
        continue;
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
      la_batch_plan_destroy(pl);
      rows.push_back({c, w, t});
      if (t < best_t) { best_t = t; best_c = c; best_w = w; }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rows.empty()) return LA_UNSUPPORTED;
  if (table_path) {
    FILE* f = fopen(table_path, "a");
    if (f) {
      for (auto& r : rows)
        fprintf(f, "%s %d %.1f %d %d %.4f\n", mode == LA_BATCH_FP64 ? "fp64" : "mixed", count,
                mean_n, r.c, r.w, r.ms);
      fclose(f);
    }
  }
  *best_ctas_per_sm = best_c;
  if (best_warps_per_system) *best_warps_per_system = best_w;
  if (best_ms) *best_ms = best_t;
  return la_sync_and_check(ctx, "batch autotune");
}

}  // extern "C"
