/*
 * matgb.h -- GB300 extensions to the mat.h API.
 *
 * None of these have a counterpart in the reference (libmat is a synchronous
 * host library with no device, stream or error channel); each says which
 * reference routine it generalises.  Everything here is C ABI: plain
 * pointers, sizes and integer status codes.  Functions named *_dev take
 * DEVICE pointers (column-major, explicit leading dimension) and are
 * asynchronous on the library stream; everything else is synchronous.
 * Status: 0 on success, < 0 on error (message in matgb_last_error()).
 */
#ifndef MATGB_H_
#define MATGB_H_

#include "mat.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Status codes -------------------------------------------------------- */
#define MATGB_OK 0
#define MATGB_ERR_CUDA (-1)     /* a CUDA call failed (message recorded)     */
#define MATGB_ERR_ARG (-2)      /* bad size / pointer / option               */
#define MATGB_ERR_NOMEM (-3)    /* device allocation failed                  */
#define MATGB_ERR_TIMEOUT (-4)  /* a bounded device wait gave up             */
#define MATGB_ERR_NOT_SPD (-5)  /* Cholesky met a diagonal <= 0              */
#define MATGB_ERR_NO_DEVICE (-6)

/* ---- Runtime ------------------------------------------------------------- */
/* Select the device and create the library stream (called implicitly by the
 * first API call with device 0).  The reference has no device state; this is
 * the GPU counterpart of its scratch-arena initialisation (mat.h:865-895). */
int matgb_init(int device);
/* Element size of this build: 4 (libmatgb_f32) or 8 (libmatgb_f64). */
int matgb_elem_size(void);
/* Last error message ("" if none) and clear.  The void mat_* functions have
 * no error channel in the reference; they record here and, unless
 * matgb_set_abort_on_error(0) was called, print and abort like MAT_ASSERT. */
const char *matgb_last_error(void);
void matgb_clear_error(void);
void matgb_set_abort_on_error(int on);
/* Wait for all work on the library stream. */
int matgb_sync(void);
/* The library stream (a cudaStream_t). */
void *matgb_stream(void);
/* Kernels launched by this library since load (host-side counter). */
unsigned long long matgb_launch_count(void);
/* Number of SMs on the current device. */
int matgb_sm_count(void);
/* Directory of the loaded library file ("" if unknown). */
const char *matgb_library_dir(void);

/* ---- Memory helpers for device-resident callers ------------------------- */
void *matgb_device_alloc(size_t bytes);
int matgb_device_free(void *p);
void *matgb_host_alloc(size_t bytes); /* page-locked host memory */
int matgb_host_free(void *p);
int matgb_memcpy_h2d(void *dst, const void *src, size_t bytes); /* async */
int matgb_memcpy_d2h(void *dst, const void *src, size_t bytes); /* async */
int matgb_memcpy_d2d(void *dst, const void *src, size_t bytes); /* async */
int matgb_memset_dev(void *dst, int value, size_t bytes);       /* async */

/* ---- Timing on the library stream (CUDA events, 16 slots) --------------- */
int matgb_event_record(int slot);
/* Milliseconds between two recorded slots (synchronises on slot1). */
double matgb_event_elapsed_ms(int slot0, int slot1);

/* Per-kernel timing: while enabled, every library launch is bracketed by
 * CUDA events on the library stream and tagged with its algorithmic FLOPs
 * and bytes.  matgb_ktime_get(i, ...) returns the i-th kernel name with its
 * launch count, total milliseconds, FLOPs and bytes (synchronises); non-zero
 * when i is past the end.  Enabling clears previous records. */
int matgb_ktime_enable(int on);
int matgb_ktime_get(int i, char *name, int cap, long long *launches,
                    double *ms, double *flops, double *bytes);
/* The i-th timed scope in launch order: its name, start and end in
 * milliseconds from the first scope's start, and its stream (numbered by
 * first appearance: 0 is the library stream when it launched first).  A
 * timeline of the streams; synchronises the device; non-zero past the end. */
int matgb_ktime_trace(int i, char *name, int cap, double *t0_ms, double *t1_ms,
                      int *stream);
/* Peak issue rate of the SIMT FMA pipes, measured with a dependent-chain-free
 * FMA kernel: which = 0 for FP32 (FFMA), 1 for FP64 (DFMA).  TFLOP/s. */
double matgb_measure_fma_peak(int which);

/* ---- Seeded input generation on the device ------------------------------ */
/* A[i] = lo + (hi-lo)*u_i with u_i = splitmix64(seed, i) mapped to [0,1). */
int matgb_fill_uniform_dev(mat_elem_t *A, size_t count, uint64_t seed,
                           double lo, double hi);
/* A[i] ~ N(0,1) by Box-Muller over the same stream. */
int matgb_fill_normal_dev(mat_elem_t *A, size_t count, uint64_t seed);
/* A[i*lda+i] += shift for i < n. */
int matgb_add_diag_dev(mat_elem_t *A, size_t n, size_t lda, double shift);

/* ---- Device-resident hot path ------------------------------------------- */
/* C = alpha*op(A)*op(B) + beta*C, op per trans flag ('N' or 'T'); C is m x n.
 * Generalises mat__gemm_strided_ (mat.h:2719-2741) / mat_gemm. */
int matgb_gemm_dev(char transa, char transb, size_t m, size_t n, size_t k,
                   mat_elem_t alpha, const mat_elem_t *A, size_t lda,
                   const mat_elem_t *B, size_t ldb, mat_elem_t beta,
                   mat_elem_t *C, size_t ldc);
/* One triangle ('L'/'U') of C (n x n) = alpha*op(A)*op(A)^T + beta*C, with
 * trans 'N' (A n x k) or 'T' (A k x n).  Generalises mat__syrk_lower_
 * (mat.h:5474-5486), mat_syrk and mat_syrk_t. */
int matgb_syrk_dev(char uplo, char trans, size_t n, size_t k,
                   mat_elem_t alpha, const mat_elem_t *A, size_t lda,
                   mat_elem_t beta, mat_elem_t *C, size_t ldc);
/* In-place P*A = L*U with partial pivoting, the same pivot rule as
 * mat__plu_blocked_ (mat.h:4201-4289: first index of max |a|, pivots with
 * |a| < MAT_DEFAULT_EPSILON swapped but not divided by).  ipiv (device, n
 * int32) receives the row swapped into position k at step k; perm (device,
 * n int32, may be NULL) receives mat_plu's permutation: perm[i] = source row
 * of row i (mat.h:4227-4229). */
int matgb_getrf_dev(size_t n, mat_elem_t *A, size_t lda, int32_t *ipiv,
                    int32_t *perm);
/* In-place full-pivoting elimination with mat_lu's pivot rule (mat.h:
 * 4476-4574): rowpiv[k] / colpiv[k] (device, n int32) receive the row and
 * the column swapped into position k at step k (k itself for none, and for
 * a skipped step).  A holds the unit-lower L below its diagonal and U on and
 * above it.  n must be below 2^31. */
int matgb_getrf_full_dev(size_t n, mat_elem_t *A, size_t lda, int32_t *rowpiv,
                         int32_t *colpiv);
/* X (n x nrhs) = A^{-1} B from getrf output: X = B[perm] then unit-lower and
 * upper triangular solves (mat_solve's steps, mat.h:4825-4830, for many
 * columns).  B is not modified; X must not alias B. */
int matgb_getrs_dev(size_t n, size_t nrhs, const mat_elem_t *LU, size_t lda,
                    const int32_t *perm, const mat_elem_t *B, size_t ldb,
                    mat_elem_t *X, size_t ldx);
/* In-place lower Cholesky of A (upper triangle not referenced).  info
 * (device int32) gets 0, or j+1 for the first column j whose diagonal was
 * <= 0 (mat.h:6046-6048 returns -1 there). */
int matgb_potrf_dev(size_t n, mat_elem_t *A, size_t lda, int32_t *info);
/* B <- A^{-1} B from the potrf factor: L y = b then L^T x = y
 * (mat_solve_spd's steps, mat.h:4862-4865).  Skips all work when *info != 0
 * (info may be NULL). */
int matgb_potrs_dev(size_t n, size_t nrhs, const mat_elem_t *L, size_t lda,
                    mat_elem_t *B, size_t ldb, const int32_t *info);
/* Triangular solve with many right-hand sides, in place on B (n x nrhs):
 * uplo 'L'/'U', trans 'N'/'T', diag 'N'/'U'.  Covers mat_solve_tril ('L','N',
 * 'N'), _tril_unit ('L','N','U'), _triu ('U','N','N') and _trilt ('L','T',
 * 'N'), mat.h:4580-4803.  Non-unit diagonals are divided by, as there. */
int matgb_trsm_dev(char uplo, char trans, char diag, size_t n, size_t nrhs,
                   const mat_elem_t *T, size_t ldt, mat_elem_t *B, size_t ldb);
/* Plain float products on the tensor cores: with on = 1 (the default) the
 * float build runs mat_mul / mat_gemm / mat_syrk (and the *_dev forms) of at
 * least 256 x 256, and the SYRK updates of mat_chol / mat_solve_spd (and
 * matgb_potrf_dev) from order 1024 up, as FP32-accurate tensor-core
 * products: each operand split into
 * FP16 hi + remainder under power-of-two row / column scales, three products
 * accumulated in FP32 (about 22 bits of every operand).  0: the FP32 SIMT
 * kernels.  -1: query only.  Returns the previous setting.  No effect in
 * libmatgb_f64.  No counterpart in the reference (its GEMM is the NEON /
 * scalar mat_gemm, mat.h:2470-2796). */
int matgb_plain_tensor_core(int on);
/* Householder QR in place: R (m x n, m >= n, leading dimension ldr) holds A
 * on entry and R on return; Q (m x m, leading dimension ldq) receives the
 * orthogonal factor, or is not formed when NULL (mat_qr_r).  Device form of
 * mat_qr / mat_qr_r (mat.h:3907-4192). */
int matgb_qr_dev(size_t m, size_t n, mat_elem_t *R, size_t ldr, mat_elem_t *Q,
                 size_t ldq);
/* y = alpha*A*x + beta*y (A m x n).  Generalises mat_gemv (mat.h:2137). */
/* y (n) = beta*y + alpha*A^T x for A m x n (mat_gemv_t, mat.h:2224-2248);
 * rows are split into chunks, summed in a fixed order, when n is small. */
int matgb_gemv_t_dev(size_t m, size_t n, mat_elem_t alpha, const mat_elem_t *A,
                     size_t lda, const mat_elem_t *x, mat_elem_t beta,
                     mat_elem_t *y);
/* y += alpha*x (mat_axpy, mat.h:2009-2015), bit-identical to the reference. */
int matgb_axpy_dev(size_t n, mat_elem_t alpha, const mat_elem_t *x,
                   mat_elem_t *y);
int matgb_gemv_dev(size_t m, size_t n, mat_elem_t alpha, const mat_elem_t *A,
                   size_t lda, const mat_elem_t *x, mat_elem_t beta,
                   mat_elem_t *y);

/* ---- Mixed precision: tensor-core LU + iterative refinement -------------- */
/* Generalises mat_solve (mat.h:4807-4837): the LU runs with FP32 panels and
 * FP32 trailing matrix, its trailing updates (mat.h:4277-4283) on the tensor
 * cores in BF16 or FP16 with FP32 accumulation; the residual, correction
 * update and convergence test run on the GPU in the library's element type
 * (FP64 in libmatgb_f64). */
typedef struct {
  int lp_format;     /* 2 (default) = FP16 split: both operands scaled by
                        powers of two and split into FP16 hi + remainder,
                        three tensor-core products per update (FP32-level
                        factors; refinement converges to kappa ~ 1e6 and
                        beyond); 3 = three-part FP16 split (hi + mid +
                        remainder, six products, ~33 bits of each operand,
                        per-row / per-column scales; LU only, the Cholesky
                        takes 2); 0 = FP16 (one product, U12 scaled);
                        1 = BF16 (one product; at n ~ 1e4 too coarse to
                        refine past kappa ~ 1e2); -1 = FP32 SIMT updates    */
  int max_iter;      /* factor solves over all attempts (default 100)        */
  double tol;        /* target backward error; <= 0: n * unit roundoff of the
                        element type (n * 2^-53 in libmatgb_f64)             */
  int fp32_fallback; /* 1 (default): if refinement with the 16-bit factors
                        stagnates, refactor once with FP32 trailing updates
                        and refine again                                     */
  int krylov;        /* 1 (default): a single right-hand side is refined by
                        flexible GMRES preconditioned with the low-precision
                        factors (converges for kappa(A) * u_16 well above 1);
                        0: classic refinement, one factor solve per step    */
  int krylov_dim;    /* Krylov vectors per cycle (default 50, at most 64)   */
} MatIROpts;

typedef struct {
  int iterations;        /* factor solves done (1 = no refinement needed)    */
  int converged;         /* backward_error <= tol                             */
  int lp_format;         /* format of the factors that produced x           */
  double backward_error; /* |b - A x|_inf / (|A|_inf |x|_inf + |b|_inf)      */
  double residual_inf, x_inf, a_inf, b_inf, tol;
  double ms_factor;      /* GPU time of conversion + factorisation(s)         */
  double ms_refine;      /* GPU time of solves, residuals and updates         */
  int refinements;       /* residuals computed in the element type            */
  int krylov_steps;      /* FGMRES steps over all cycles (0: classic)         */
  double forward_error_est; /* the solver's own estimate of the forward
                        error |x - x*|_inf / |x*|_inf (it has no exact
                        solution to compare with): one right-hand side
                        (FGMRES): |M^-1 r|_inf / |x|_inf, the correction the
                        low-precision factors M give for the final residual
                        r; many right-hand sides (classic refinement): the
                        largest |d|_inf / |x|_inf of the last correction d,
                        an upper estimate (it is the error of the iterate
                        before that correction)                            */
} MatIRReport;

void matgb_ir_default_opts(MatIROpts *o);
/* Solve A x = b (device pointers, A n x n column-major). */
int matgb_gesv_ir_dev(size_t n, const mat_elem_t *A, size_t lda,
                      const mat_elem_t *b, mat_elem_t *x,
                      const MatIROpts *opts, MatIRReport *rep);
/* Host Mat form; returns 0 or a negative status. */
int mat_solve_ir(Vec *x, const Mat *A, const Vec *b, const MatIROpts *opts,
                 MatIRReport *rep);
/* Many right-hand sides (B, X: n x nrhs; the backward error reported is the
 * largest over the columns). */
int matgb_gesv_ir_multi_dev(size_t n, size_t nrhs, const mat_elem_t *A,
                            size_t lda, const mat_elem_t *B, size_t ldb,
                            mat_elem_t *X, size_t ldx, const MatIROpts *opts,
                            MatIRReport *rep);
/* SPD form (generalises mat_solve_spd, mat.h:4839-4871): Cholesky of the lower
 * triangle with FP32 panels and tensor-core SYRK updates (BF16, or FP16 with a
 * power-of-two scale), refinement as above.  Returns 0, -1 when the matrix is
 * not positive definite (even in FP32), or a negative status. */
int matgb_posv_ir_dev(size_t n, size_t nrhs, const mat_elem_t *A, size_t lda,
                      const mat_elem_t *B, size_t ldb, mat_elem_t *X,
                      size_t ldx, const MatIROpts *opts, MatIRReport *rep);
/* Host Mat form of matgb_posv_ir_dev (b and x n x nrhs). */
int mat_solve_spd_ir(Vec *x, const Mat *A, const Vec *b, const MatIROpts *opts,
                     MatIRReport *rep);
/* The FP32 Cholesky alone (device, in place, lower) with tensor-core (2 FP16
 * split, 1 BF16, 0 FP16) or SIMT (-1) trailing updates; *info as
 * matgb_potrf_dev. */
int matgb_potrf_lp_dev(size_t n, float *A, size_t lda, int32_t *info,
                       int lp_format);
/* The FP32 LU alone (device, in place) with trailing updates on the tensor
 * cores (lp_format 3 three-part FP16 split, 2 FP16 split, 1 BF16, 0 FP16)
 * or, for lp_format -1, the FP32 SIMT GEMM.
 * ipiv/perm as matgb_getrf_dev.  Pivots are never skipped (threshold 0). */
int matgb_getrf_lp_dev(size_t n, float *A, size_t lda, int32_t *ipiv,
                       int32_t *perm, int lp_format);
/* R -= A X (double build only; A n x n, X and R n x nrhs, column-major) with
 * FP64-level accuracy from exact FP16 digit products on the tensor cores:
 * rows of A and columns of X are cut into 8 signed 7-bit digits under a
 * power-of-two scale, digit pairs multiplied over 1024-term chunks (exact
 * in FP32) and accumulated in FP64.  The multi-RHS refinement residual of
 * matgb_gesv_ir_multi_dev / matgb_posv_ir_dev (the step of mat.h:4820-4837
 * and 4862-4865 repeated per correction) uses it from n = 1024 up. */
int matgb_resid64_dev(size_t n, size_t nrhs, const mat_elem_t *A, size_t lda,
                      const mat_elem_t *X, size_t ldx, mat_elem_t *R, size_t ldr);
/* 0: the multi-RHS refinement forms residuals with the FP64 GEMM instead
 * (for measurement); 1 (default): digit slices on the tensor cores. */
int matgb_resid64_mode(int on);
/* C (fp32, column-major, M x N) = beta*C + alpha * A * B^T with A (M x K) and
 * B (N x K) K-contiguous BF16 (bf16 != 0) or FP16, K a multiple of 64 and at
 * most 128, lda/ldb multiples of 8: the tensor-core rank-K update
 * (tcgen05.mma, TMEM accumulators, TMA-fed) behind the mixed LU. */
int matgb_tc_gemm_dev(int bf16, size_t M, size_t N, size_t K, const void *A,
                      size_t lda, const void *B, size_t ldb, float alpha,
                      float beta, float *C, size_t ldc);
/* Split form: FP16 hi parts (Ah, Bh) and remainders (Al, Bl), same layouts;
 * computes C = beta*C + alpha*(Ah Bh^T + Ah Bl^T + Al Bh^T) in one pass over
 * C (three tensor-core products, FP32 accumulation).  K a multiple of 64. */
int matgb_tc_gemm_split_dev(size_t M, size_t N, size_t K, const void *Ah,
                            const void *Al, size_t lda, const void *Bh,
                            const void *Bl, size_t ldb, float alpha, float beta,
                            float *C, size_t ldc);
/* 0, or MATGB_ERR_TIMEOUT if a tensor-core kernel gave up a bounded wait
 * since the last call (clears the flag; synchronises). */
int matgb_tc_status(void);
/* Short-K tensor-core products (the trailing updates): 1 (default) = the
 * persistent form (two CTAs per SM pulling 128 x 128 tiles from a counter,
 * two TMEM accumulators each so a tile's epilogue runs under the next
 * tile's MMAs); 0 = one CTA per 128 x 256 tile.  -1 queries.  Returns the
 * previous setting. */
int matgb_tc_persistent(int on);
/* The mixed LU's look-ahead after a fused 144-column block (split FP16
 * update): 1 (default) = the next block's row swaps, U12 solve and both
 * operands' packing in one launch, U12 scaled per column; 0 = the separate
 * swap, solve and packing launches with one U12 scale.  -1 queries.
 * Returns the previous setting. */
int matgb_la_prep(int on);
/* The tensor-core Cholesky (mixed SPD solve, plain float Cholesky from order
 * 1024): 1 (default) = look-ahead, the diagonal block, its column solve and
 * the next block's columns on a high-priority stream while the library
 * stream updates the rest of the trailing matrix; 0 = every step in turn on
 * the library stream.  -1 queries.  Returns the previous setting. */
int matgb_chol_lookahead(int on);

/* y = alpha*A*x + beta*y like matgb_gemv_dev, for callers that must not
 * allocate device memory -- e.g. code that runs inside another runtime's
 * memory pool (where a raw cudaMalloc can fail or fragment that pool) or on a
 * latency-critical stream (where cudaMalloc/cudaFree's implicit device
 * synchronisation is not acceptable).  No counterpart in the reference.
 * Allocates nothing: its scratch is a static device array of 2^20 elements
 * (4 MiB in libmatgb_f32, 8 MiB in libmatgb_f64) that every GPU loading the
 * library holds until exit; m above 2^20 is rejected with MATGB_ERR_ARG.
 * Runs on `stream` (a cudaStream_t; NULL = the legacy default stream) and
 * does not touch the library stream.  The first call on a device looks up the
 * array's device address, so make that first call before any stream
 * capture.  All calls share the array: calls that overlap on the GPU (other
 * streams, other threads) race and must be serialised by the caller. */
int matgb_gemv_noalloc_dev(size_t m, size_t n, mat_elem_t alpha,
                           const mat_elem_t *A, size_t lda,
                           const mat_elem_t *x, mat_elem_t beta,
                           mat_elem_t *y, void *stream);

/* ---- Batched small systems ------------------------------------------------- */
/* Solve `count` independent systems in one pass (mat_solve / mat_solve_spd
 * applied to each, mat.h:4807-4871).  status[s] = -2 marks an order outside
 * 1..128 (not solved); with the fused schedule, -4 marks a system left
 * unsolved because the launch's bounded grid barrier gave up (never expected:
 * the launch is cooperative).  Device pointers: system s has order
 * n[s] (1..128), its matrix at A + offA[s]
 * (column-major, leading dimension n[s]) and its right-hand side / solution at
 * b + offv[s] / x + offv[s].  kind[s] = 0: partial-pivot LU with the
 * reference's pivot rule; 1: Cholesky of the lower triangle.  status[s]: 0, or
 * -1 when Cholesky met a pivot <= 0 (x[s] then untouched, as mat_solve_spd
 * returns -1).  Asynchronous on the library stream. */
int matgb_solve_batched_dev(int64_t count, const int32_t *n,
                            const int64_t *offA, const mat_elem_t *A,
                            const int64_t *offv, const mat_elem_t *b,
                            mat_elem_t *x, const uint8_t *kind,
                            int32_t *status);
/* The batched solver's schedule per (size bucket nb = 16, 32, 64, 96 or 128,
 * kind 0 general / 1 SPD): algo 0 = one row per thread, Gauss-Jordan with one
 * barrier per column; 1 = blocked LU in 8-column panels (nb >= 64);
 * ctas_per_sm caps the resident systems per SM (0: as many as fit).  The
 * library starts from compiled-in defaults, then reads the tuner's file
 * (libmat_gb300/batched_tune.json next to the library directory, or
 * $LIBMATGB_BATCHED_TUNE) at the first batched call; this call overrides
 * one entry.  No counterpart in the reference. */
int matgb_batched_tune(int nb, int kind, int algo, int ctas_per_sm);
int matgb_batched_tune_get(int nb, int kind, int *algo, int *ctas_per_sm);
/* The batched solver's launch schedule: fused = 1 files and
 * solves every system in ONE persistent cooperative launch (orders 65..128
 * one per CTA, 33..64 two, 17..32 four, 1..16 eight; largest first), 0 = one
 * launch per (bucket, kind) queue with the per-bucket algorithms above;
 * ctas_per_sm caps the fused launch's resident CTAs per SM (0: as many as
 * fit); graphs = 1 (the default) captures either launch sequence in a CUDA
 * graph and replays it while the same buffers are passed.  The compiled-in
 * default is fused = 0 (measured faster on the 100k-system workload); the
 * tuner's file may choose.  -1 leaves a setting unchanged.  Returns the
 * previous fused setting. */
int matgb_batched_schedule(int fused, int ctas_per_sm, int graphs);
/* Where the schedule came from: "defaults" or the file and its entry count. */
const char *matgb_batched_tune_source(void);
/* The mixed-precision batched mode (float build only).  A queue of orders
 * 33..128 that it routes to the tensor-core kernels is solved with the
 * matrix held in tensor memory, blocked Gauss-Jordan in 32-column panels
 * whose transforms and trailing updates run as TF32 hi + remainder products
 * with FP32 accumulation (~21 bits), then FP32 residuals and corrections
 * until the normwise backward error |r|/(|A||x| + |b|) <= n 2^-24 (at most 4
 * corrections).  Its status[s] is then 0 (converged), 1 (not converged: x
 * holds the last iterate), -1 (an SPD pivot <= 0, x untouched) or -3 (a wait
 * for the tensor core gave up).  A general system keeps the diagonal pivots
 * when, in every panel, partial pivoting would keep them within the 32-row
 * pivot block and the panel's transform entries stay within 1; otherwise it
 * is factored again with partial pivoting (on the values this factorisation
 * computes, so the pivots may differ from the reference's on near-ties).
 * on = 1: the queues chosen per (bucket, kind) by matgb_batched_mixed_tune /
 * the tuner's file (compiled-in: general 97..128); on = 2: every queue of
 * orders 33..128; 0: off (the FP32 kernels only, the reference's
 * semantics).  Queues not routed keep the FP32 kernels.  on = -1 only
 * queries.  Returns the previous setting (an error code for on > 0 in the
 * double build).  No counterpart in the reference. */
int matgb_batched_mixed(int on);
/* Route queue (nb = 64, 96 or 128, kind 0 general / 1 SPD) to the
 * tensor-core kernel (use_tc = 1) or the FP32 kernel (0) when the mixed mode
 * is 1. */
int matgb_batched_mixed_tune(int nb, int kind, int use_tc);
/* The last batched call's mixed-mode counts (synchronises the library
 * stream): refinement corrections taken, systems with status 1, and whether
 * a wait gave up.  Any pointer may be NULL. */
int matgb_batched_mixed_stats(int *corrections, int *unconverged, int *timeouts);

/* ---- Host (Mat) superset ------------------------------------------------- */
/* AX = B for every column of B (mat_solve reads only column 0, mat.h:4825). */
void matgb_solve_multi(Mat *X, const Mat *A, const Mat *B);
/* SPD variant; returns 0 or -1 like mat_solve_spd. */
int matgb_solve_spd_multi(Mat *X, const Mat *A, const Mat *B);

#ifdef __cplusplus
}
#endif

#endif /* MATGB_H_ */
