// Internal declarations shared by the liblagpu translation units.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/la_gpu.h"

// Largest device ordinal whose one-time set-up results are cached.
constexpr int LA_MAX_DEVICES = 64;

// The current CUDA device, or -1 when it cannot be read.
inline int la_current_device() {
  int dev = -1;
  return cudaGetDevice(&dev) == cudaSuccess ? dev : -1;
}

// One-time set-up per device. Kernel attributes (cudaFuncSetAttribute) and
// occupancy answers belong to the device that is current at the call, and
// several host threads (one context each) may arrive at once: each device runs
// the set-up once under the lock, later calls only read an atomic bit mask. A
// set-up that fails runs again on the next call.
struct la_device_once {
  std::mutex mu;
  std::atomic<uint64_t> done{0};
  // f(dev) returns cudaError_t; cudaSuccess when this device ran it before.
  template <typename F>
  cudaError_t run(F&& f) {
    const int dev = la_current_device();
    if (dev < 0) return cudaErrorInvalidDevice;
    std::unique_lock<std::mutex> lock(mu, std::defer_lock);
    if (dev >= LA_MAX_DEVICES) {  // not cached: set up on every call
      lock.lock();
      return f(dev);
    }
    const uint64_t bit = 1ull << dev;
    if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
    lock.lock();
    if (done.load(std::memory_order_relaxed) & bit) return cudaSuccess;
    cudaError_t e = f(dev);
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_release);
    return e;
  }
};

// Accumulation forms of the FP64 kernels.
//  FAST : c = fma(-a, b, c)                      (blocked LU, in place)
//  EXACT: the reference's order, no fusion:
//         LU carry  s = s + a*b, value = x - s   (lu.rs:122-128)
//         solve     x = x - a*b per term         (lu.rs:260, :272)
enum GemmMode : int {
  GM_FMA_SUB = 0,        // C = C - A*B   fused, ascending k
  GM_FMA_ZERO = 1,       // C = A*B       fused, from zero
  GM_EXACT_ADD = 2,      // C = C + a*b   unfused, ascending k (LU carry)
  GM_EXACT_ZERO = 3,     // C = 0 + a*b   unfused, ascending k (Mul, mod.rs:965-973)
  GM_EXACT_SUB = 4,      // C = C - a*b   unfused, ascending k (forward solve)
  GM_EXACT_SUB_DESC = 5, // C = C - a*b   unfused, descending k (back solve)
  GM_FMA_SUB_DESC = 6    // C = C - A*B   fused, descending k
};

constexpr int MAX_PANEL_CTAS = 1024;
constexpr int MAX_PANEL_W = 64;
// Column groups (4 right-hand sides each) of the wavefront triangular solve;
// more right-hand sides take the block-step solve.
constexpr int SOLVE_WAVE_MAX_GROUPS = 1024;

// Device-side error codes written to la_context::d_err.
enum DeviceErr : int {
  DERR_NONE = 0,
  DERR_PANEL_TIMEOUT = 1,
  DERR_PANEL_CAPACITY = 2,
  DERR_TC_TIMEOUT = 3,
  DERR_TRSV_TIMEOUT = 4,
  DERR_GEMM_TIMEOUT = 5
};

// Operand formats of the tensor-core update. The split formats store each
// value as a high and a low part (v ~ hi + lo) and accumulate the three
// products hi*hi + hi*lo + lo*hi: LA_LOWP_E4M3X3 in FP8 e4m3 (about BF16
// accuracy), LA_LOWP_F16X3 in FP16 (about 2^-22 per product, near FP32).
enum LowpFormat : int { LA_LOWP_BF16 = 1, LA_LOWP_FP16 = 2, LA_LOWP_E4M3X3 = 3, LA_LOWP_F16X3 = 4 };

struct la_context {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t side_stream = nullptr;    // high priority: lookahead panels
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  int lookahead = 1;
  int cluster_panels = 1;                // FP32 panels on one thread-block cluster
  int batch_gmres = 0;                   // Krylov steps per GMRES correction in batch plans (0: off)
  int solve_wave = 2;                    // CTAs per SM of the wavefront solve (0: block steps)
  int inject_alloc_at = 0;               // the n-th device allocation from now fails (0: none)
  int inject_ir_stall = 0;               // this many refinement calls report a stall at once
  int inject_panel_stall = 0;            // the n-th FP64 panel launch from now waits for a CTA too many
  long long wait_limit_us = 0;           // limit of the panel's grid-barrier wait (0: 2 s)
  int sm_count = 0;
  size_t smem_optin = 0;
  int arith = LA_ARITH_FAST;
  int panel_width = 64;
  int panel_ctas = 0;
  int profile = 0;
  int pdl = 1;                           // LA_OPT_PDL: dependent launches in the mixed LU's panel chain
  bool pdl_now = false;                  // set while that chain is being enqueued
  std::string last_error;
  uint64_t launches = 0;
  double phase_ms[5] = {0, 0, 0, 0, 0};
  std::vector<cudaEvent_t> event_pool;  // reused by the per-phase timer

  // Device scratch for the cooperative panel kernel and small results.
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  int* d_err = nullptr;          // inside d_scratch
  unsigned* d_bar = nullptr;     // barrier counters (one per panel)
  size_t bar_count = 0;
  int cand_stride = MAX_PANEL_CTAS;  // candidate slots per parity in the buffers below
  double* d_cand_abs = nullptr;  // [2][MAX_PANEL_CTAS]
  int* d_cand_pos = nullptr;     // [2][MAX_PANEL_CTAS]
  double* d_cand_row = nullptr;  // [2][MAX_PANEL_CTAS][64]
  double* d_diag_a = nullptr;    // [2][64]
  double* d_diag_s = nullptr;    // [2][64]
  int* d_swaps = nullptr;        // [1 + 2*128] composed row moves of one panel
  double* d_small = nullptr;     // [8] small device results (det, flags)
  int* d_solve_sync = nullptr;   // [2 + 2*SOLVE_WAVE_MAX_GROUPS] wavefront solve tickets, progress
  void* h_pinned = nullptr;      // pinned host staging for small readbacks
};

struct la_lu_handle {
  la_ctx ctx = nullptr;
  size_t m = 0, n = 0, ld = 0;
  double* d_lu = nullptr;
  int* d_ipiv = nullptr;         // LAPACK-style swap list, absolute rows, length min(m,n)
  uint64_t* d_piv = nullptr;     // permutation vector (lu.rs piv), length m
  int pospivsign = 1;
  int zero_diag = 0;             // an exact 0 on U's diagonal (j < min(m,n))
  int arith = LA_ARITH_FAST;
  // Mixed-precision factorization: FP32 factors (d_lu32, pitch ld32) of the
  // FP64 matrix kept in d_lu (used for residuals); null for plain FP64.
  float* d_lu32 = nullptr;
  size_t ld32 = 0;
  double* d_dinv = nullptr;      // inverted 64x64 diagonal blocks of L and U (lazy, FP64)
  float* d_dinvf = nullptr;      // the same in FP32 (plain refinement)
  int lowp = 0;                  // LA_PREC_* of the trailing update
};


// Programmatic dependent launch. A kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization (la_launch with
// ctx->pdl_now set) may be scheduled while the kernel before it on the stream
// still runs; la_pdl_wait blocks until that kernel has completed and its
// writes are visible, so every such kernel calls it before touching global
// memory. la_pdl_trigger lets the next kernel be scheduled once every CTA of
// this one has passed it. Both return at once in a kernel launched without
// the attribute.
__device__ __forceinline__ void la_pdl_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void la_pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launches kernel k on stream s, as a programmatic dependent launch when
// ctx->pdl_now is set.
template <typename... KArgs, typename... Args>
cudaError_t la_launch(la_ctx ctx, void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                      cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  if (ctx->pdl_now) {
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// Host helpers (context.cu).
la_status la_cuda_fail(la_ctx ctx, cudaError_t e, const char* what);
la_status la_check_launch(la_ctx ctx, const char* what);
la_status la_device_alloc(la_ctx ctx, void** p, size_t bytes);
void la_device_free(la_ctx ctx, void* p);
la_status la_sync_and_check(la_ctx ctx, const char* what);

#define LA_TRY(expr)                       \
  do {                                     \
    la_status _s = (expr);                 \
    if (_s != LA_OK) return _s;            \
  } while (0)

#define LA_CUDA(ctx, call)                                  \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return la_cuda_fail(ctx, _e, #call); \
  } while (0)

// Kernel launchers (one per translation unit of kernels).
la_status launch_tc_update(la_ctx ctx, cudaStream_t stream, int fmt, int M, int N, int K,
                           const void* A, size_t lda, const void* B, size_t ldb, float* C,
                           size_t ldc, const float* d_alpha);
// min_smem > 0 raises the GEMM's dynamic shared memory so fewer CTAs share an
// SM (room for a concurrent panel CTA).
la_status launch_gemm(la_ctx ctx, int mode, int M, int N, int K, const double* A, size_t lda,
                      const double* B, size_t ldb, double* C, size_t ldc, size_t min_smem = 0);
// C -= A B on the 64 x 64 output tiles at or below the diagonal of the square
// C (M x M, FMA); LA_UNSUPPORTED (nothing launched) where TMA cannot take the
// operands.
la_status launch_gemm_lower(la_ctx ctx, int M, int K, const double* A, size_t lda,
                            const double* B, size_t ldb, double* C, size_t ldc);
// C + z * czs = A[:, z kper : (z + 1) kper] B[z kper : (z + 1) kper, :] for z < splits
// (fused, from zero); kper a multiple of 32, splits * kper >= K > (splits - 1) kper.
la_status launch_gemm_splitk(la_ctx ctx, int M, int N, int K, const double* A, size_t lda,
                             const double* B, size_t ldb, double* C, size_t ldc, size_t czs,
                             int splits, int kper);
// Blocked FAST QR (qr_blocked.cu): blocks of QR_BLOCK columns in compact WY
// form. qr_blocked_factor factors A (m x n, pitch ld) in place, writes rdiag
// and each block's Gram matrix V'V (QR_BLOCK x QR_BLOCK, one after another) to
// gram; LA_UNSUPPORTED (nothing launched) when the rows exceed one cluster's
// shared memory. qr_blocked_apply applies the factored reflections to T:
// mode 1 (get_q) Q[j:, j:] block by block in reverse, mode 2 (solve) X[j:, :]
// in order; cols = T's columns.
constexpr int QR_BLOCK = 64;
bool qr_blocked_supported(la_ctx ctx, int m, int n);
la_status qr_blocked_factor(la_ctx ctx, double* A, size_t ld, int m, int n, double* rdiag,
                            double* gram);
la_status qr_blocked_apply(la_ctx ctx, const double* A, size_t ld, int m, int dc,
                           const double* rdiag, const double* gram, int mode, double* T,
                           size_t ldt, int cols);
la_status launch_panel(la_ctx ctx, cudaStream_t stream, bool exact, double* A, double* S,
                       size_t ld, int m, int j0, int jb, int* d_ipiv, unsigned* bar_base);
la_status launch_laswp(la_ctx ctx, bool exact, double* A, double* S, size_t ld, int n, int j0,
                       int jb);
la_status launch_trsm_rowpanel(la_ctx ctx, bool exact, double* A, double* S, size_t ld, int j0,
                               int jb, int c_begin, int c_end);
la_status launch_panel_f32(la_ctx ctx, cudaStream_t stream, float* A, size_t ld, int m, int j0,
                           int jb, int* d_ipiv, unsigned* bar_base);
la_status launch_laswp_f32(la_ctx ctx, float* A, size_t ld, int n, int j0, int jb);
la_status launch_laswp_seq_f32(la_ctx ctx, float* A, size_t ld, const int* ipiv, int k0, int k1,
                               int c0, int c1);
la_status launch_panel_cluster_f32(la_ctx ctx, float* A, size_t ld, int m, int j0, int jb,
                                   int* d_ipiv);
la_status launch_trsm_rowpanel_f32(la_ctx ctx, float* A, size_t ld, int j0, int jb, int c_begin,
                                   int c_end);
// X = L11^-1 X for rows [j0, j0 + jbo) (jbo <= 256) of columns [c_begin, c_end).
la_status launch_trsm_block_f32(la_ctx ctx, float* A, size_t ld, int j0, int jbo, int c_begin,
                                int c_end);
la_status launch_gemm_f32(la_ctx ctx, int mode, int M, int N, int K, const float* A, size_t lda,
                          const float* B, size_t ldb, float* C, size_t ldc);
la_status launch_lu_solve_f32(la_ctx ctx, const float* LU, size_t ld, float* X, size_t ldx, int n,
                              int nrhs);
la_status launch_invert_diag_f32(la_ctx ctx, const float* LU, size_t ld, int n, double* dinv);
la_status launch_trsv_wave_f32(la_ctx ctx, const float* LU, size_t ld, const double* dinv,
                               double* X, size_t ldx, int n, int nrhs, int* sync);
la_status launch_invert_diag_f32f(la_ctx ctx, const float* LU, size_t ld, int n, float* dinv);
la_status launch_trsv_wave_f32f(la_ctx ctx, const float* LU, size_t ld, const float* dinv,
                                float* X, size_t ldx, int n, int nrhs, int* sync);
la_status launch_lu_finish(la_ctx ctx, la_lu h, int* d_flags);
// Enqueues the whole factorization of h (no readback, no synchronization);
// lu_finish writes {pospivsign, zero-on-diagonal} to d_flags.
la_status lu_factor_enqueue(la_ctx ctx, la_lu h, int* d_flags);
la_status launch_tri_wave(la_ctx ctx, bool exact, bool upper, bool divide, const double* T,
                          size_t ld, double* X, size_t ldx, int n, int nrhs);
la_status launch_lu_solve(la_ctx ctx, bool exact, const double* LU, size_t ld, double* X,
                          size_t ldx, int n, int nrhs);
la_status launch_permute_rows(la_ctx ctx, const uint64_t* d_piv, const double* B, size_t ldb,
                              double* X, size_t ldx, int m, int nrhs);
la_status launch_identity_permuted(la_ctx ctx, const uint64_t* d_piv, double* X, size_t ldx,
                                   int m);
la_status launch_det(la_ctx ctx, const double* LU, size_t ld, int n, int pospivsign,
                     double* d_out);
la_status launch_unpack(la_ctx ctx, int which, const double* LU, size_t ld, int m, int n,
                        const uint64_t* d_piv, double* out);
la_status launch_copy2d(la_ctx ctx, const double* src, size_t lds, double* dst, size_t ldd,
                        int rows, int cols);
