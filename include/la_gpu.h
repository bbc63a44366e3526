/*
 * la_gpu.h — C ABI of the GB300 (sm_103a) dense LU factor-and-solve library
 * (liblagpu.so). It is the drop-in boundary for the LU path of the `la` crate
 * (xasmx/rust-la 0.2.0): a Rust, C, C++ or Python host binds these symbols and
 * keeps the crate's types and semantics on its side.
 *
 * Conventions shared by every entry point:
 *  - Matrices are dense, row-major f64, exactly like Matrix<f64>'s Vec<f64>
 *    (src/matrix/mod.rs:26-30). Host pointers are plain (pageable or pinned)
 *    memory; *_device entry points take device pointers with a row pitch `ld`
 *    in elements.
 *  - The reference's `assert!` failures (a panic) come back as LA_BADSHAPE and
 *    its `None` as LA_SINGULAR. Nothing is written to the outputs then.
 *  - Host-pointer calls return when their results are in host memory. Device
 *    calls are ordered on the context's stream; an LU handle is complete when
 *    la_lu_new* returns (pivots, sign and the singular flag are read back).
 *  - One context serves one host thread at a time (the reference is
 *    single-threaded); use one context per thread for concurrency.
 */
#ifndef LA_GPU_H
#define LA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LA_ABI_VERSION 1

typedef enum la_status {
  LA_OK = 0,
  LA_SINGULAR = 1,       /* reference returns None (exact zero on U's diagonal) */
  LA_BADSHAPE = 2,       /* reference panics (failed assert! / index out of bounds) */
  LA_INVALID = 3,        /* null handle/pointer, bad option value */
  LA_NOMEM = 4,          /* device or pinned allocation failed */
  LA_CUDA_ERROR = 5,     /* a CUDA runtime call failed; see la_ctx_last_error */
  LA_TIMEOUT = 6,        /* a bounded device-side wait gave up; the context stays usable */
  LA_NOT_CONVERGED = 7,  /* iterative refinement stalled (mixed-precision entry points) */
  LA_UNSUPPORTED = 8     /* size or option outside what this build implements */
} la_status;

typedef struct la_context* la_ctx;
typedef struct la_lu_handle* la_lu;
typedef struct la_chol_handle* la_chol;
typedef struct la_qr_handle* la_qr;

/* ---- context ------------------------------------------------------------ */

/* Creates a context on CUDA device `device` with its own non-blocking stream. */
la_status la_ctx_create(int device, la_ctx* out);
void la_ctx_destroy(la_ctx ctx);
/* Orders all later work of this context on `stream` (a cudaStream_t); NULL
 * restores the context's own stream. */
la_status la_ctx_set_stream(la_ctx ctx, void* stream);
void* la_ctx_get_stream(la_ctx ctx);
la_status la_ctx_synchronize(la_ctx ctx);
const char* la_status_string(la_status s);
/* Message of the last LA_CUDA_ERROR / LA_TIMEOUT seen by this context. */
const char* la_ctx_last_error(la_ctx ctx);
int la_abi_version(void);

/* Options (la_ctx_set_option). */
typedef enum la_option {
  /* LU arithmetic. LA_ARITH_FAST (default): blocked right-looking LU with
   * fused multiply-add. LA_ARITH_EXACT: the same blocked kernels carry each
   * element's partial sum separately and add terms in the reference's order
   * without fusion, so LU factors, pivots, det and solve results are
   * bit-identical to src/decomp/lu.rs (at about half the FP64 rate). Also
   * selects the summation of la_matrix_mul (mod.rs:957-980 order when EXACT). */
  LA_OPT_ARITH = 1,
  /* Panel width of the blocked LU (16, 32 or 64). */
  LA_OPT_PANEL_WIDTH = 2,
  /* Upper bound on CTAs of the cooperative panel kernel (0 = all SMs). */
  LA_OPT_PANEL_CTAS = 3,
  /* 1: record per-phase device times of each LU (la_ctx_last_phase_ms). */
  LA_OPT_PROFILE = 4,
  /* 1 (default): factor the next panel on a second stream while the rest of
   * the trailing update runs; 0: strictly one phase after the other. */
  LA_OPT_LOOKAHEAD = 5,
  /* 1 (default): the FP32 panels of the mixed LU run on one thread-block
   * cluster (distributed shared memory); 0: the cooperative multi-CTA kernel. */
  LA_OPT_CLUSTER_PANEL = 6,
  /* Batch plans (read when a plan is built): largest Krylov basis (0-20) of
   * the GMRES-IR stage that a LA_BATCH_MIXED plan runs on a system whose
   * LU-IR reached a backward error below 1e-6 and then stalled, before the
   * FP64 pass; 0 (default) turns the stage off. It pays off for factors whose
   * LU-IR contracts but slowly (BF16 / FP8 storage of well-conditioned
   * systems); with FP32 factors the stalled systems have kappa u_32 near 1 and
   * need more Krylov steps than the FP64 redo costs. */
  LA_OPT_BATCH_GMRES = 7,
  /* Triangular solves of la_lu_solve (lu.rs:256-275): 1-8 (default 2) runs
   * them as one persistent wavefront kernel per triangle with that many CTAs
   * per SM; 0 launches one kernel per 16-row block step. Both apply every
   * term in the same order, so their results are bit-identical. */
  LA_OPT_SOLVE_WAVE = 8,
  /* Failure injection on the host, for tests (0 = off; reads back what is
   * left). INJECT_ALLOC_FAIL = k: the k-th device allocation of this context
   * from now returns LA_NOMEM, as an exhausted pool would. INJECT_IR_STALL = k:
   * the next k refinement calls (la_lu_solve_refined_device and each stage of
   * la_lu_solve_auto_device) report a stall before their first correction. */
  LA_OPT_INJECT_ALLOC_FAIL = 10,
  LA_OPT_INJECT_IR_STALL = 11,
  /* Limit, in microseconds, of the grid-barrier wait of the cooperative panel
   * kernel (1 to 10,000,000; 0 = the default of 2 s). A CTA whose wait runs
   * out records the failure and returns, every other CTA sees it and returns,
   * the kernels queued behind the panel that would use its row interchanges
   * return at entry, and the call reports LA_TIMEOUT; the context stays
   * usable. */
  LA_OPT_WAIT_LIMIT_US = 12,
  /* Failure injection for tests (0 = off; reads back what is left): the k-th
   * launch of the cooperative panel kernel from now makes its CTAs wait for
   * one arrival more than there are CTAs, so that the wait runs out (after
   * LA_OPT_WAIT_LIMIT_US) exactly as when a CTA cannot reach the barrier. */
  LA_OPT_INJECT_PANEL_STALL = 13,
  /* 1 (default): in the mixed LU, the chain of inner-panel kernels (32-column
   * panel, row swaps, triangular solve, rank-32 update) and the serial part
   * between outer panels (row swaps, the next panel's triangular solve, U12
   * scale and packing, tensor-core update) are launched with programmatic
   * stream serialization, so that each kernel is scheduled while the one
   * before it finishes and waits on the device for its results; 0: ordinary
   * stream order. Results are bit-identical either way. */
  LA_OPT_PDL = 14
} la_option;

#define LA_ARITH_FAST 0
#define LA_ARITH_EXACT 1

la_status la_ctx_set_option(la_ctx ctx, int option, int64_t value);
la_status la_ctx_get_option(la_ctx ctx, int option, int64_t* value);

/* ---- LUDecomposition<f64> (src/decomp/lu.rs) ---------------------------- */

/* LUDecomposition::new (lu.rs:104-168). Copies A (m x n, m,n > 0) to the
 * device and factors it with partial pivoting. Never reports LA_SINGULAR
 * (the reference's `new` always succeeds). */
la_status la_lu_new(la_ctx ctx, const double* a, size_t m, size_t n, la_lu* out);
/* Same, from device memory (row pitch lda >= n elements). */
la_status la_lu_new_device(la_ctx ctx, const double* d_a, size_t lda, size_t m, size_t n,
                           la_lu* out);
void la_lu_free(la_lu lu);
la_status la_lu_shape(la_lu lu, size_t* m, size_t* n);

/* lu.rs:170-182. *out = 1 when non-singular. LA_BADSHAPE where the
 * reference indexes past its data (m < n with no zero diagonal found first). */
la_status la_lu_is_non_singular(la_lu lu, int* out);
/* lu.rs:224-232: (+-1) * product of U's diagonal in ascending order.
 * LA_BADSHAPE unless square. */
la_status la_lu_det(la_lu lu, double* out);
/* lu.rs:222 get_piv (a permutation: piv[i] = original row now at i) and the
 * sign flag (lu.rs:99). Either pointer may be NULL. */
la_status la_lu_get_piv(la_lu lu, uint64_t* piv, int* pospivsign);
/* The packed m x n LU (lu.rs:98): unit-L below the diagonal, U on/above. */
la_status la_lu_get_packed(la_lu lu, double* out);
/* lu.rs:184-202: m x min(m,n). */
la_status la_lu_get_l(la_lu lu, double* out);
/* lu.rs:204-215: min(m,n) x n. */
la_status la_lu_get_u(la_lu lu, double* out);
/* lu.rs:217-220: m x m permutation matrix, row i = e_{piv[i]}. */
la_status la_lu_get_p(la_lu lu, double* out);
/* Device pointer and row pitch of the packed LU (valid while `lu` lives). */
const double* la_lu_device_data(la_lu lu, size_t* ld);

/* LUDecomposition::solve (lu.rs:237-278). B is brows x nrhs; X is m x nrhs.
 * LA_BADSHAPE if brows != m, LA_SINGULAR if U has an exact zero diagonal. */
la_status la_lu_solve(la_lu lu, const double* b, size_t brows, size_t nrhs, double* x);
/* Same on device memory (pitches ldb, ldx >= nrhs). */
la_status la_lu_solve_device(la_lu lu, const double* d_b, size_t ldb, size_t brows,
                             size_t nrhs, double* d_x, size_t ldx);

/* ---- Matrix<f64> methods that go through LU (src/matrix/mod.rs) ---------- */

/* mod.rs:1025-1028: asserts square, LU, det. */
la_status la_matrix_det(la_ctx ctx, const double* a, size_t m, size_t n, double* out);
/* mod.rs:1030-1032: LUDecomposition::new(a).solve(b) (no square assert). */
la_status la_matrix_solve(la_ctx ctx, const double* a, size_t m, size_t n, const double* b,
                          size_t brows, size_t nrhs, double* x);
/* mod.rs:1034-1037: asserts square, then LU.solve(Matrix::id(n, n)). */
la_status la_matrix_inverse(la_ctx ctx, const double* a, size_t m, size_t n, double* out);
/* mod.rs:1044-1047: asserts square, LU, is_non_singular. */
la_status la_matrix_is_non_singular(la_ctx ctx, const double* a, size_t m, size_t n, int* out);

/* ---- Matrix * Matrix (mod.rs:957-998, mmatrix.rs:82-98) ------------------ */

/* C (m x n) = A (m x k) * B (brows x n). LA_BADSHAPE unless k == brows. */
la_status la_matrix_mul(la_ctx ctx, const double* a, size_t m, size_t k, const double* b,
                        size_t brows, size_t n, double* c);
/* mmul: like la_matrix_mul into a caller buffer of dst_rows x dst_cols;
 * LA_BADSHAPE unless dst is m x n (mmatrix.rs:83-85). */
la_status la_matrix_mmul(la_ctx ctx, const double* a, size_t m, size_t k, const double* b,
                         size_t brows, size_t n, double* dst, size_t dst_rows, size_t dst_cols);
/* Device form: C = A * B with row pitches; stream-ordered, no sync. */
la_status la_matrix_mul_device(la_ctx ctx, const double* d_a, size_t lda, const double* d_b,
                               size_t ldb, double* d_c, size_t ldc, size_t m, size_t k, size_t n);

/* ---- mixed precision + iterative refinement (no reference counterpart) ---- */

/* Precision of the trailing-update products of the mixed LU. */
#define LA_PREC_BF16 1  /* tcgen05 BF16 x BF16 -> FP32 */
#define LA_PREC_FP16 2  /* tcgen05 FP16 x FP16 -> FP32, per-panel power-of-two scaling */
#define LA_PREC_FP32 3  /* FP32 FMA (no tensor cores) */
/* mixed LU: tcgen05 FP8 e4m3 with each operand split in a high and a low part
 * (three products, about BF16 accuracy); batched solves: factors stored as FP8
 * e4m3 (power-of-two scaled) */
#define LA_PREC_FP8 4
#define LA_PREC_FP64 5  /* batched solves: no mixed attempt, the plan's FP64 pass answers */
/* mixed LU: tcgen05 FP16 x FP16 -> FP32 with each operand split in a high and
 * a low FP16 part (three products, about 2^-22 relative error each: factors
 * close to FP32 ones at the cost of the FP16 update) */
#define LA_PREC_FP16X3 6

typedef struct la_refine_stats {
  int iterations;    /* refinement steps (plain and GMRES) */
  int converged;     /* 1 when eta <= tol was reached */
  double eta;        /* final normwise backward error (FP64 residual) */
  int fell_back;     /* 1 when the plain FP64 LU produced the answer */
  int precision;     /* LA_PREC_* actually used for the answer (0: plain FP64) */
  int gmres_steps;   /* Arnoldi steps of GMRES-IR (0: plain refinement sufficed) */
} la_refine_stats;

/* Factors a square FP64 matrix (device, pitch lda) in FP32 with the trailing
 * updates in `prec`; the handle keeps the FP64 matrix for residuals. Pivoting
 * is partial pivoting on the FP32 values. */
la_status la_lu_mixed_new_device(la_ctx ctx, const double* d_a, size_t lda, size_t n, int prec,
                                 la_lu* out);
/* Iterative refinement with the mixed factors: x = 0, r = b; d = LU \ r (FP32),
 * x += d, r = b - A x (FP64) until eta <= tol. When that stalls it continues
 * with GMRES-IR (GMRES on M^-1 A d = M^-1 r, M the low-precision LU) until
 * eta <= tol, max_iters steps in all, or a stall (LA_NOT_CONVERGED).
 * nrhs <= 16. */
la_status la_lu_solve_refined_device(la_lu lu, const double* d_b, size_t ldb, size_t nrhs,
                                     double* d_x, size_t ldx, int max_iters, double tol,
                                     la_refine_stats* stats);
/* Solves A X = B (A n x n FP64 on the device, B and X n x nrhs, nrhs <= 16)
 * to a normwise backward error <= tol: (1) the mixed LU with split-FP16
 * trailing updates (LA_PREC_FP16X3: FP32-quality factors at the FP16
 * update's cost), plain refinement and then GMRES-IR, at most 40 steps;
 * (2) the plain FP64 LU and solve (LUDecomposition::new + solve,
 * lu.rs:104-278), which answers whatever (1) could not.
 * stats->precision is LA_PREC_FP16X3 or 0 (plain FP64, then
 * stats->fell_back = 1), stats->iterations the refinement steps of all stages
 * and stats->eta the final backward error. LA_SINGULAR only when the plain
 * FP64 LU has an exact zero pivot (the reference's None). No reference
 * counterpart: it replaces Matrix::solve (mod.rs:1030-1032) for callers that
 * accept any factorization whose answer meets tol. */
la_status la_lu_solve_auto_device(la_ctx ctx, const double* d_a, size_t lda, size_t n,
                                  const double* d_b, size_t ldb, size_t nrhs, double* d_x,
                                  size_t ldx, double tol, la_refine_stats* stats);
/* Tensor-core building block of the mixed LU, exposed for testing:
 * C (m x n f32, pitch ldc) -= alpha * A (m x k) * B^T (B: n x k), K-major.
 * fmt 1 = BF16, 2 = FP16: pitches multiples of 8 elements. Split formats,
 * fmt 3 = FP8 e4m3 (bytes) and 4 = FP16: each row holds the high parts in
 * columns [0, k) and the low parts from column lda / 2 (lda == ldb, lda / 2 at
 * or beyond k rounded up to 128 bytes, pitches multiples of 32 bytes); the
 * kernel accumulates Ah Bh^T + Ah Bl^T + Al Bh^T. */
la_status la_lowp_update_device(la_ctx ctx, int fmt, size_t m, size_t n, size_t k,
                                const void* d_a16, size_t lda, const void* d_b16, size_t ldb,
                                float* d_c, size_t ldc, float alpha);

/* ---- batched solves of many small systems (no reference counterpart) ----- */

/* One system of a batch: A at d_a + a_offset (n x n, row-major FP64), B and X
 * at d_b / d_x + b_offset (n x nrhs, row-major FP64); 1 <= n <= 512,
 * 1 <= nrhs <= 4. `precision` (mixed batches) is the storage of its LU
 * factors: LA_PREC_FP8, LA_PREC_BF16 or LA_PREC_FP32 (0 = FP32); arithmetic is
 * FP32 either way, and narrower storage lets larger systems stay in shared
 * memory at the cost of less accurate factors. LA_PREC_FP64 sends the system
 * straight to the plan's FP64 pass (no mixed attempt). */
typedef struct la_batch_system {
  size_t a_offset;
  size_t b_offset;
  int n;
  int nrhs;
  int precision;
  int reserved;
} la_batch_system;

#define LA_BATCH_FP64 0   /* plain FP64 LU + solve per system */
#define LA_BATCH_MIXED 1  /* low-precision LU + FP64 refinement, FP64 redo where it stalls */

typedef struct la_batch_plan_s* la_batch_plan;

/* Builds the work queue (systems sorted by decreasing n), the scratch, and a
 * CUDA graph holding the whole batch: one persistent fused factor + solve
 * launch (plus, for LA_BATCH_MIXED, the FP64 pass over systems whose
 * refinement did not reach `tol` within `max_iters`). Each system is worked by
 * one CTA of 32 * warps_per_system threads (2, 4 or 8; 0 = 8); ctas_per_sm
 * (1-8) such CTAs share an SM and its shared memory, and a system whose
 * layout does not fit its CTA's share works with its matrix in global
 * scratch. LA_UNSUPPORTED when the largest system cannot fit even so, or when
 * ctas_per_sm CTAs of that size cannot be resident on one SM. The plan runs
 * once while it is built. */
la_status la_batch_plan_create(la_ctx ctx, const double* d_a, const double* d_b, double* d_x,
                               const la_batch_system* systems, int count, int mode,
                               int ctas_per_sm, int warps_per_system, double tol, int max_iters,
                               la_batch_plan* out);
/* Launches the plan's graph on the context's stream (asynchronous). */
la_status la_batch_plan_run(la_batch_plan plan);
/* Per system (caller's order): refinement steps, final backward error (-1 when
 * the FP64 kernel produced the answer), and 1 when the FP64 pass redid it.
 * Any pointer may be NULL. Synchronizes. */
la_status la_batch_plan_stats(la_batch_plan plan, int* iterations, double* eta, int* fell_back);
void la_batch_plan_destroy(la_batch_plan plan);
/* Splits a batch (caller's order) into `parts` contiguous slices of about
 * equal cost for `parts` GPUs, one plan per GPU over its slice and no
 * collective in the plans: the cost of system i is its LU and solve flops,
 * 2/3 n^3 + 2 n^2 nrhs, and bounds[p] (parts + 1 ints, bounds[0] = 0,
 * bounds[parts] = count, non-decreasing) is the system where the cumulative
 * cost comes nearest to p / parts of the total; slice p is systems
 * [bounds[p], bounds[p + 1]). Host only, no context. */
la_status la_batch_partition(const la_batch_system* systems, int count, int parts, int* bounds);
/* Autotuner: times every supported (ctas_per_sm, warps_per_system) pair in
 * {1, 2, 4, 8} x {8, 4, 2} on this batch and returns the fastest; appends
 * "mode count mean_n ctas_per_sm warps_per_system ms" lines for all candidates
 * to table_path when it is not NULL. best_warps_per_system may be NULL. */
la_status la_batch_autotune(la_ctx ctx, const double* d_a, const double* d_b, double* d_x,
                            const la_batch_system* systems, int count, int mode, double tol,
                            int max_iters, const char* table_path, int* best_ctas_per_sm,
                            int* best_warps_per_system, double* best_ms);

/* Sets each system's factor storage from d_class (device, caller's order, one
 * int per system: 0 = FP8, 1 = BF16, 2 = FP32, the classes of the precision
 * selector, or 3 = no mixed attempt, straight to the FP64 pass) for the
 * following runs of a LA_BATCH_MIXED plan, without rebuilding it;
 * asynchronous on the context's stream. */
la_status la_batch_plan_select_device(la_batch_plan plan, const int* d_class);
/* Row order of the factorization that produced each system's X in the last
 * run (lu.rs:147-149 piv: piv[i] = the original row at position i): the FP64
 * pass's for systems it answered, the mixed pass's otherwise. piv (host) holds
 * sum of n_i entries, the systems one after the other in the caller's order.
 * Synchronizes. */
la_status la_batch_plan_pivots(la_batch_plan plan, uint64_t* piv);
/* Phase profile of the last run: SM cycles summed over all CTAs, phase[0..3]
 * = load (and FP8 scaling), factorization, triangular solves, residuals and
 * convergence tests of the first pass; phase[4..7] the same for the FP64 redo
 * pass of a LA_BATCH_MIXED plan. Synchronizes. */
la_status la_batch_plan_phase_cycles(la_batch_plan plan, long long* phase);
/* Per system (caller's order): SM clock cycles its CTA spent on it in the last
 * run, summed over the mixed and the FP64 pass. Synchronizes. */
la_status la_batch_plan_cycles(la_batch_plan plan, long long* cycles);

/* ---- learned precision selector (no reference counterpart) --------------- */

/* 16 features per system (row-major FP32 [count][16]) for the precision
 * selector: log2 n / 9, nrhs / 4, log10 of the max row and column sums, of the
 * Frobenius norm, of max |a_ij|, of the 4-step Lanczos estimate of sigma_max,
 * of ||A||_F / sigma_max, of the smallest diagonal-dominance ratio, the mean
 * log10 dominance ratio, the fraction of dominant rows, log10 of the row-sum
 * and column-sum spreads, the asymmetry probe ||A q - A^T q|| / ||A q|| (q the
 * fixed Lanczos start vector),
 * log10 min|a_ii| / max|a_ij|, and log10 of the Lanczos estimate of
 * sigma_max / sigma_min (a lower bound on kappa_2). Systems as in a batch
 * plan (1 <= n <= 512); synchronizes. */
la_status la_batch_features_device(la_ctx ctx, const double* d_a, const la_batch_system* systems,
                                   int count, float* d_features);

/* Householder-conditioned test systems: A_i = H1 diag(s) H2 with
 * s_k = kappa_i^(-k/(n-1)), log10 kappa_i uniform in [log10_kappa_min,
 * log10_kappa_max], H1 and H2 products of four random reflectors, B_i iid
 * N(0,1); all seeded (counter-based, reproducible). d_kappa (count doubles)
 * may be NULL. Synchronizes. */
la_status la_generate_conditioned_batch(la_ctx ctx, const la_batch_system* systems, int count,
                                        double log10_kappa_min, double log10_kappa_max,
                                        unsigned long long seed, double* d_a, double* d_b,
                                        double* d_kappa);

/* MLP 16 -> 64 -> 64 -> 3 (ReLU, softmax; FP32) over the classes
 * 0 = LA_PREC_FP8, 1 = LA_PREC_BF16, 2 = LA_PREC_FP32. Parameters, in order:
 * W1[64][16], b1[64], W2[64][64], b2[64], W3[3][64], b3[3]
 * (la_mlp_param_count() floats), then the feature means[16] and standard
 * deviations[16] the inputs are normalised with. */
typedef struct la_mlp_s* la_mlp;
int la_mlp_param_count(void);
la_status la_mlp_create(la_ctx ctx, unsigned long long seed, la_mlp* out);
void la_mlp_destroy(la_mlp mlp);
/* params: la_mlp_param_count() + 32 floats (host). Setting resets Adam. */
la_status la_mlp_get_params(la_mlp mlp, float* params);
la_status la_mlp_set_params(la_mlp mlp, const float* params);
/* Mean softmax cross-entropy over count samples (d_x [count][16], d_y labels
 * 0..2, device) and its gradient (host, la_mlp_param_count() floats; NULL to
 * skip); no update. Synchronizes. */
la_status la_mlp_gradients(la_mlp mlp, const float* d_x, const int* d_y, int count, float* grad,
                           float* loss);
/* One Adam step (beta 0.9 / 0.999) on the mean cross-entropy of the samples;
 * loss (host, may be NULL) is taken before the step and synchronizes. */
la_status la_mlp_train_step(la_mlp mlp, const float* d_x, const int* d_y, int count, float lr,
                            float* loss);
/* The same two calls for the expected cost instead of the cross-entropy:
 * d_cost [count][3] (device) holds each sample's cost of the three classes
 * (e.g. measured cycles, scaled), and the loss is the mean over the samples
 * of sum_c p_c cost_c, so that training weighs each system by what a wrong
 * class costs it rather than counting mistakes. */
la_status la_mlp_gradients_cost(la_mlp mlp, const float* d_x, const float* d_cost, int count,
                                float* grad, float* loss);
la_status la_mlp_train_step_cost(la_mlp mlp, const float* d_x, const float* d_cost, int count,
                                 float lr, float* loss);
/* Class probabilities (d_probs [count][3], may be NULL) and argmax classes
 * (d_class, may be NULL; 3 where the gate below sends the system straight to
 * the FP64 pass); asynchronous on the context's stream. */
la_status la_mlp_predict(la_mlp mlp, const float* d_x, int count, float* d_probs, int* d_class);
/* Gate of la_mlp_predict's classes: with coef (19 floats) set, a system whose
 * score coef[0..15] . x + coef[16..18] . p + bias >= 0 (x its raw, unnormalised
 * features, p its three class probabilities) gets class 3, no mixed attempt
 * (la_batch_plan_select_device sends it straight to the FP64 pass). coef NULL
 * turns the gate off (the default). LA_INVALID for non-finite values. */
la_status la_mlp_set_gate(la_mlp mlp, const float* coef, float bias);

/* ---- allocation-free factorization (no reference counterpart) ------------ */

/* LU factorization (FAST arithmetic) for callers that cannot allocate device
 * memory, e.g. code whose device memory is owned by a pool or framework that
 * forbids cudaMalloc, or that must keep a fixed footprint. It allocates
 * nothing and needs no la_ctx: it factors d_a (m x n, row-major, pitch lda,
 * 16-byte aligned, lda even) in place on `stream` (a cudaStream_t, NULL for
 * the default stream) and writes the swap list d_ipiv (min(m,n) int32), the
 * permutation vector d_piv (m uint64, the form of lu.rs piv) and d_flags[0] =
 * pospivsign, d_flags[1] = 1 if U has an exact zero on its diagonal.
 * The call blocks until the stream has finished the factorization (it waits on
 * the stream and reads the device error word with a synchronous copy), so it
 * cannot be called while any stream is being captured into a CUDA graph.
 * Limit: m <= 16384 (LA_UNSUPPORTED beyond). Its working memory is one static
 * device array of about 70 KB per device, kept until the process exits and
 * shared by every call: calls that overlap on the GPU (other host threads,
 * other streams) race and must be serialized by the caller. The first call on
 * a device looks up that array's device address; after cudaDeviceReset that
 * address is stale and the library must not be called again in the process.
 * Status: LA_INVALID for null pointers, lda < n, or d_a not 16-byte aligned or
 * lda odd; LA_BADSHAPE for m or n = 0; LA_UNSUPPORTED beyond the limit (or a
 * panel that does not fit the kernel's shared memory); LA_TIMEOUT when any
 * bounded device wait of the factorization (panel barrier, TMA stage of the
 * trailing update) gave up; LA_CUDA_ERROR when a CUDA call failed. There is no
 * context, so no message is kept beyond the status. */
la_status la_lu_factor_noalloc(void* stream, double* d_a, size_t lda, size_t m, size_t n,
                               int* d_ipiv, uint64_t* d_piv, int* d_flags);

/* ---- accuracy check (no reference counterpart) --------------------------- */

/* Normwise backward error of a computed solution X of A X = B (A n x n):
 *   eta = max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf),
 * with the residual accumulated in compensated FP64 on the device. */
la_status la_backward_error_device(la_ctx ctx, const double* d_a, size_t lda, const double* d_x,
                                   size_t ldx, const double* d_b, size_t ldb, size_t n,
                                   size_t nrhs, double* eta);
la_status la_backward_error(la_ctx ctx, const double* a, const double* x, const double* b,
                            size_t n, size_t nrhs, double* eta);
/* The same for every system of a batch (systems as in la_batch_plan_create,
 * any n >= 1 and nrhs >= 1): d_eta[i] (device, count doubles, caller's order)
 * is system i's eta, computed with the same compensated FP64 residual; when
 * max_eta (host) is not NULL it receives the largest of them (NaN if any is
 * NaN). Synchronizes. */
la_status la_batch_backward_error_device(la_ctx ctx, const double* d_a, const double* d_b,
                                         const double* d_x, const la_batch_system* systems,
                                         int count, double* d_eta, double* max_eta);

/* ---- Cholesky decomposition (src/decomp/cholesky.rs) ------------------------ */

/* CholeskyDecomposition::new (cholesky.rs:56-111): A (m x n, row-major host
 * memory) = L L'. LA_OK with *out set, or LA_SINGULAR with *out = NULL where
 * the reference returns None: A not square (:57-59), A[k][j] != A[j][k] for
 * some k < j (:89-91, so a NaN off the diagonal too), or A[j][j] - d <= 0 at
 * some row (:97-100). LA_BADSHAPE for m == 0 or n == 0 (Matrix::new asserts).
 * LA_OPT_ARITH = LA_ARITH_EXACT gives L bit-identical to the reference;
 * LA_ARITH_FAST (default) uses FMA and a blocked order. */
la_status la_chol_new(la_ctx ctx, const double* a, size_t m, size_t n, la_chol* out);
/* The same from an n x n device matrix with pitch lda (elements). */
la_status la_chol_new_device(la_ctx ctx, const double* d_a, size_t lda, size_t n, la_chol* out);
void la_chol_free(la_chol c);
la_status la_chol_n(la_chol c, size_t* n);
/* CholeskyDecomposition::get_l (cholesky.rs:113): L, n x n row-major host
 * memory, zeros above the diagonal. */
la_status la_chol_get_l(la_chol c, double* out);
/* CholeskyDecomposition::solve (cholesky.rs:116-145): x (n x nrhs host) with
 * A x = b. LA_BADSHAPE where the reference's assert! panics (brows != n). */
la_status la_chol_solve(la_chol c, const double* b, size_t brows, size_t nrhs, double* x);
/* The same on device memory (pitches ldb, ldx in elements). */
la_status la_chol_solve_device(la_chol c, const double* d_b, size_t ldb, size_t brows,
                               size_t nrhs, double* d_x, size_t ldx);

/* ---- QR decomposition (src/decomp/qr.rs) ------------------------------------ */

/* QRDecomposition::new (qr.rs:26-105): Householder reflections, one column at
 * a time, on A (m x n host memory); LA_BADSHAPE for m == 0 or n == 0. EXACT
 * arithmetic gives the reference's bits (factors, Q, solution). */
la_status la_qr_new(la_ctx ctx, const double* a, size_t m, size_t n, la_qr* out);
la_status la_qr_new_device(la_ctx ctx, const double* d_a, size_t lda, size_t m, size_t n,
                           la_qr* out);
void la_qr_free(la_qr qr);
/* is_full_rank (qr.rs:108-115); LA_BADSHAPE where the reference indexes past
 * its min(m, n) diagonal (n > m and no zero among the first m). */
la_status la_qr_is_full_rank(la_qr qr, int* out);
/* get_h (qr.rs:119-132) and get_r (:135-148): m x n; get_q (:151-194): m x m. */
la_status la_qr_get_h(la_qr qr, double* out);
la_status la_qr_get_r(la_qr qr, double* out);
la_status la_qr_get_q(la_qr qr, double* out);
/* solve (qr.rs:199-238): x (n x nrhs). LA_SINGULAR where it returns None (not
 * full rank); LA_BADSHAPE where it panics: brows != m (:200), the rank test's
 * out-of-bounds index, or m != n (Matrix::new's length assert, :237). The
 * reference's arithmetic is kept, which for a general A is not A^-1 b: its
 * Q'B step divides by -u_k where its reflection uses a * u_k. */
la_status la_qr_solve(la_qr qr, const double* b, size_t brows, size_t nrhs, double* x);
/* Matrix::pinverse (mod.rs:1049-1057): (R'R)^-1 A' (n x m); LA_BADSHAPE where
 * inverse() is None and unwrap panics. */
la_status la_matrix_pinverse(la_ctx ctx, const double* a, size_t m, size_t n, double* out);

/* ---- SVD::direct (src/decomp/svd.rs) ---------------------------------------- */

/* SVD::direct (svd.rs:454-497) of A (m x n, row-major host memory):
 * u (m x m), s (m x n, the singular values on its diagonal, descending) and
 * v (n x n) with A = U S V' (to rounding). A'A and A V S^-1 run on the GPU
 * (la_matrix_mul), S^-1 by the GPU LU inverse; the eigendecomposition of A'A
 * (EigenDecomposition::new, eigen.rs:755-790: tred2 + tql2) runs on the host,
 * as in the reference. For m > n the last m - n columns of U are zero, as the
 * reference computes them; for m < n the SVD of A' is taken and U and V swap
 * (:458-466). LA_OPT_ARITH = LA_ARITH_EXACT gives the reference's bits.
 * LA_BADSHAPE where the reference panics: m or n = 0, or a zero singular value
 * (s.inverse().unwrap() on None, :483). LA_UNSUPPORTED where A'A holds a NaN
 * (the reference's nonsymmetric eigen branch, not built) or the QL iteration
 * does not converge (non-finite data; the reference's loop would not end). */
la_status la_svd_direct(la_ctx ctx, const double* a, size_t m, size_t n, double* u, double* s,
                        double* v);

/* ---- reading matrices (src/util.rs) ----------------------------------------- */

/* util::read_csv (util.rs:9-35) with the f64 parser s.parse::<f64>().unwrap():
 * the comma-separated file at `path` as a new row-major rows x cols matrix in
 * host memory (release it with la_host_free). Lines end at '\n' (a '\r' before
 * it is dropped), items are split at ',' and trimmed of Unicode white space,
 * and each must be a Rust f64 literal (sign, digits with an optional '.',
 * optional exponent; or inf, infinity, nan in any case), rounded to nearest.
 * LA_BADSHAPE where the reference panics: the file cannot be opened or is not
 * UTF-8, an item does not parse, a line has another item count than the first
 * (:25-27), or the file has no line (:32). No context or GPU is involved. */
la_status la_read_csv_f64(const char* path, double** data, size_t* rows, size_t* cols);
void la_host_free(void* p);

/* ---- diagnostics ---------------------------------------------------------- */

/* Measures this GPU's FP64 FMA issue rate (TFLOP/s) with a short all-SM
 * register-resident loop; used as the roofline denominator for FP64 kernels. */
la_status la_probe_fp64_peak(la_ctx ctx, double* tflops);
/* Number of kernels this context launched since creation (for launch counts). */
uint64_t la_ctx_kernel_launches(la_ctx ctx);
/* Per-phase device time of the last LU factorization, in milliseconds
 * (panel, row swaps, triangular update, trailing GEMM, other), measured with
 * CUDA events when LA_OPT_PROFILE is set; zeros otherwise. */
la_status la_ctx_last_phase_ms(la_ctx ctx, double* ms5);

#ifdef __cplusplus
}
#endif
#endif /* LA_GPU_H */
