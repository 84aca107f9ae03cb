// Internal declarations shared by the libmatgb translation units.
// Every TU is compiled twice: default (float) and -DMAT_DOUBLE_PRECISION.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mat.h"
#include "matgb.h"

namespace mgb {

using elem_t = mat_elem_t;

// Pivot skip threshold of the reference's LU (mat.h:4235, MAT_DEFAULT_EPSILON).
constexpr elem_t kPivotEps = (elem_t)MAT_DEFAULT_EPSILON;

struct Ctx {
  int device = -1;
  int sms = 0;
  int cluster16 = 0;  // non-portable 16-CTA clusters usable for the LU panel
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[16] = {};
};

// Lazily initialised context (device 0 unless matgb_init chose another).
Ctx *ctx();

// Route the library's launches to another stream for a scope (the panel
// streams of the look-aheads).
struct StreamSwap {
  cudaStream_t saved;
  explicit StreamSwap(cudaStream_t s) : saved(ctx()->stream) { ctx()->stream = s; }
  ~StreamSwap() { ctx()->stream = saved; }
};

// Record an error; returns `code`.  Never aborts (callers decide).
int set_error(int code, const char *fmt, ...);
// Record a CUDA failure with its call site.
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);
int launch_check(const void *func, const char *name, size_t smem);
// For the void mat_* entry points: report and abort unless disabled.
void fail_void(const char *where);

// Host-side launch accounting + launch-error check.
int launched(const char *name);
// The counter itself (a CUDA graph replay adds its kernels by hand; a
// capture, which launches nothing, is taken back out).
unsigned long long launch_counter();
void launch_counter_set(unsigned long long v);

// Optional per-kernel timing (matgb_ktime_enable): a scope records CUDA events
// on the library stream around one launch and tags it with the launch's
// algorithmic FLOPs and bytes.  Costs nothing when disabled.
struct KtScope {
  int idx;
  KtScope(const char *name, double flops, double bytes);
  ~KtScope();
};
bool ktime_on();

// Grow-only device buffers keyed by slot, reused across calls (the device
// counterpart of the reference's scratch arena, mat.h:865-895).
enum WsSlot {
  WS_A = 0, WS_B, WS_C, WS_X, WS_L, WS_U, WS_PIV, WS_INFO,
  WS_T0, WS_T1, WS_T2, WS_T3, WS_V0, WS_V1, WS_K, WS_KV, WS_RS, WS_SWM, WS_SWG,
  WS_RZA, WS_RZB, WS_RZC, WS_RZE, WS_TCA, WS_TCB, WS_TCS, WS_QR,
  // the mixed look-ahead's U12 column scales and L21 scale (la_prep)
  WS_LAS,
  // the tensor-core trailing update's packing buffers, one set per side
  // stream of a chunked factorisation (set 0 is WS_T0..WS_T2)
  WS_CU0,
  WS_NSLOTS = WS_CU0 + 3 * 8
};
void *ws(int slot, size_t bytes);

}  // namespace mgb

#define MGB_CUDA(call)                                                         \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return mgb::cuda_fail(e_, #call, __FILE__, __LINE__);                    \
  } while (0)

#define MGB_TRY(expr)                                                          \
  do {                                                                         \
    int r_ = (expr);                                                           \
    if (r_ != 0) return r_;                                                    \
  } while (0)

#define MGB_LAUNCHED(name)                                                     \
  do {                                                                         \
    int r_ = mgb::launched(name);                                              \
    if (r_ != 0) return r_;                                                    \
  } while (0)

// Internal device-pointer routines shared between TUs (all async on the
// library stream; sizes as int64 to keep index math 64-bit).
namespace mgb {
int gemm(bool ta, bool tb, int64_t m, int64_t n, int64_t k, elem_t alpha,
         const elem_t *A, int64_t lda, const elem_t *B, int64_t ldb,
         elem_t beta, elem_t *C, int64_t ldc, int tri /*0 full,1 L,2 U*/);
// Same, but every CTA returns at once when *skip != 0 (skip may be null).
int gemm_skip(bool ta, bool tb, int64_t m, int64_t n, int64_t k, elem_t alpha,
              const elem_t *A, int64_t lda, const elem_t *B, int64_t ldb,
              elem_t beta, elem_t *C, int64_t ldc, int tri,
              const int32_t *skip);
int gemv(int64_t m, int64_t n, elem_t alpha, const elem_t *A, int64_t lda,
         const elem_t *x, elem_t beta, elem_t *y);
// Element-type templates (float and double are instantiated in every build;
// the mixed-precision solvers use the float ones inside the double library).
template <typename T>
int gemm_skip_t(bool ta, bool tb, int64_t m, int64_t n, int64_t k, T alpha,
                const T *A, int64_t lda, const T *B, int64_t ldb, T beta, T *C,
                int64_t ldc, int tri, const int32_t *skip);
template <typename T>
int gemv_t(int64_t m, int64_t n, T alpha, const T *A, int64_t lda, const T *x,
           T beta, T *y);
template <typename T>
int trsm_left_t(bool lower, bool trans, bool unit, int64_t n, int64_t nrhs,
                const T *Tm, int64_t ldt, T *B, int64_t ldb,
                const int32_t *info);
struct SwapMap;
// keep (may be null): also leave the block's net swap map there
template <typename T>
int laswp_t(T *A, int64_t lda, int64_t c0, int64_t c1, int64_t c2, int64_t c3,
            const int32_t *ipiv, int64_t k1, int64_t k2, int32_t *perm,
            SwapMap *keep = nullptr);
template <typename T>
int lu_panel_t(T *A, int64_t lda, int64_t n, int64_t k0, int w, int32_t *ipiv,
               T eps, int *w_used);
// Columns of the matrix arriving in chunks while it is factored: chunk k
// (columns [k*cw, (k+1)*cw), cw a multiple of the outer block) is in the
// matrix once ev[k] has completed.  Chunk 0 is waited for before the first
// block.  Chunk k >= 1 catches up on a side stream of its own -- the row
// swaps, U12 solve and trailing update of each finished block applied to its
// columns, block after block, the same operations in another order -- and
// joins the main stream's updates just before the look-ahead reaches its
// first block.
constexpr int kMaxChunks = 64;
struct ArrivalPlan {
  int nchunks = 0;
  int64_t cw = 0;
  cudaEvent_t ev[kMaxChunks] = {};
};
// lp: -1 = trailing updates by the SIMT GEMM in T; 0 = FP16, 1 = BF16
// tensor-core updates (T = float only; FP32 panels and trailing matrix).
// arr (may be null): the columns arrive in chunks (see ArrivalPlan).
template <typename T>
int getrf_t(int64_t n, T *A, int64_t lda, int32_t *ipiv, int32_t *perm, T eps,
            int lp, const ArrivalPlan *arr = nullptr);
// Tensor-core trailing update of columns [c0,c1) after outer block [kb,ke)
// (mixed.cu): packs U12[:, c0:c1] to 16 bits, and L21 too on the block's
// first call (first = true).
// amax3 (may be null): the block's max slots [|L21|, |U12| look-ahead, |U12|
// rest], zeroed once per factorisation; l21_ready / u12_ready: already filled
// by the factorisation kernels.
// wset: the packing buffers' set (0: the main stream's; s >= 1: side
// stream s of a chunked factorisation).
int lp_trailing_update(int64_t n, float *A, int64_t lda, int64_t kb,
                       int64_t ke, int64_t c0, int64_t c1, int lp, bool first,
                       unsigned *amax3 = nullptr, bool l21_ready = false,
                       bool u12_ready = false, int wset = 0);
// y = beta*y + alpha*A^T x and y += alpha*x (blas_t.cu).
template <typename T>
int gemv_t_t(int64_t m, int64_t n, T alpha, const T *A, int64_t lda,
             const T *x, T beta, T *y);
template <typename T>
int axpy_t(int64_t n, T alpha, const T *x, T *y);
// Full-pivoting elimination (lu_full.cu); rowpiv/colpiv (device, n int32):
// the row and column swapped into position k at step k.
template <typename T>
int getrf_full_t(int64_t n, T *A, int64_t lda, int32_t *rowpiv,
                 int32_t *colpiv, T eps);
template <typename T>
int getrs_t(int64_t n, int64_t nrhs, const T *LU, int64_t lda,
            const int32_t *perm, const T *B, int64_t ldb, T *X, int64_t ldx);
// Tensor-core rank-K update (tc_gemm.cu).
// lower: only tiles on/below the diagonal, elements with col <= row;
// skip: every CTA returns at once when *skip != 0 (may be null);
// Alo/Blo (may be null): remainders of A and B for the three-product split.
// lower: 0 every element, 1 lower triangle, 2 upper triangle (tiles and
// elements outside it are skipped); rinv/cinv (may be null): per-row and
// per-column power-of-two factors applied to the product before alpha (rinv
// only together with cinv); persist: 1 the persistent short-K form, 0 one
// CTA per tile (its CTAs retire tile by tile, so that kernels of a
// higher-priority stream find SMs meanwhile), -1 the library setting.
int tc_gemm(int bf16, int64_t M, int64_t N, int64_t K, const void *A,
            int64_t lda, const void *B, int64_t ldb, float alpha,
            const float *alpha_scale, float beta, float *C, int64_t ldc,
            int lower, const int32_t *skip, const void *Alo = nullptr,
            const void *Blo = nullptr, const float *rinv = nullptr,
            const float *cinv = nullptr, const void *Amid = nullptr,
            const void *Bmid = nullptr, int persist = -1);
// FP32-accurate float GEMM / SYRK on the tensor cores (tc_sgemm.cu): op(A)
// and op(B) packed to FP16 hi + remainder under per-row / per-column
// power-of-two scales, three products per update; tri as tc_gemm's lower.
// parts 3: hi + mid + remainder, six products (about 33 bits of each
// operand: the FP32 products' own rounding is then the larger error).
int tc_sgemm(bool ta, bool tb, int64_t m, int64_t n, int64_t k, float alpha,
             const float *A, int64_t lda, const float *B, int64_t ldb,
             float beta, float *C, int64_t ldc, int tri, bool same_ab = false,
             int parts = 2);
// Whether the plain float paths (GEMM, SYRK, Cholesky) use the tensor cores
// (matgb_plain_tensor_core), and the size from which they do.
bool plain_tc_on();
constexpr int64_t kPlainTcMinMN = 256;
constexpr int64_t kPlainTcMinN = 1024;  // Cholesky order
// FP64 residual R -= A X (X n x nrhs) on the tensor cores from exact FP16
// digit products (resid64.cu); resid64_prepare slices A once per solve.
int resid64_prepare(int64_t n, const double *A, int64_t lda);
int resid64(int64_t n, int64_t nrhs, const double *A, const double *X, int64_t ldx,
            double *R, int64_t ldr);
// Cholesky trailing update C22 -= L21 L21^T on the tensor cores (mixed.cu).
int lp_syrk_update(int64_t m, int nb, const float *L21, int64_t lda,
                   float *C22, int64_t ldc, int lp, const int32_t *info);
// The same in two steps: L21 packed once (buffer set 0 or 1), then any
// lower-triangular block of the product applied (C relative to its origin:
// rows [r0, r0+M) of the operand against rows [c0, c0+N)).
struct SyrkOperand {
  uint16_t *hi, *lo;  // m x Kp, K-contiguous; lo null unless split
  float *sc;          // scale slots: [0] s, [1] 1/s, [2] 1/s^2
  int Kp;
  int64_t m;
  int lp;
};
// amax_ready: the set's max slot (lp_syrk_amax_slot) already holds max|L21|.
int lp_syrk_pack(int64_t m, int nb, const float *L21, int64_t lda, int lp, int set,
                 SyrkOperand *op, bool amax_ready = false);
unsigned *lp_syrk_amax_slot(int set);
int lp_syrk_apply(const SyrkOperand &op, int64_t r0, int64_t M, int64_t c0, int64_t N,
                  float *C, int64_t ldc, const int32_t *info, int persist = -1);
template <typename T>
int potrf_t(int64_t n, T *A, int64_t lda, int32_t *info, int lp);
// Single-launch triangular solve with one right-hand side (trsv.cu); inv
// (float only): diagonal sub-blocks through explicit inverses, for the
// refinement's preconditioner.
template <typename T>
int trsv_t(bool lower, bool trans, bool unit, int64_t n, const T *Tm,
           int64_t ldt, T *x, bool inv = false);
// The low-precision factors applied to one vector (the FGMRES
// preconditioner): out = (P^T L U)^-1 in (LU) or (L L^T)^-1 in (spd).
int precond_solve(bool spd, int64_t n, const float *W, const int32_t *perm,
                  const float *in, float *out);
int trsv_status();
// Triangular solve with many right-hand sides in one launch per 64 columns
// (trsm_flag.cu); trsm_flag_status() reports a bounded wait that gave up.
template <typename T>
int trsm_flag_t(bool lower, bool trans, bool unit, int64_t n, int64_t nrhs,
                const T *Tm, int64_t ldt, T *B, int64_t ldb, const int32_t *info);
int trsm_flag_status();
template <typename T>
int potrs_t(int64_t n, int64_t nrhs, const T *L, int64_t lda, T *B,
            int64_t ldb, const int32_t *info);
int tc_error_flag(int clear);
// 1 when an LU panel's column exchange gave up waiting (lu.cu); read after a
// stream synchronisation.
int lu_wait_error(int clear);
// Flexible GMRES for the refinement correction (krylov.cu): solves A d = r0
// with r0 in V(:, 0) on entry; V holds m + 1 and Z m vectors of length n, F
// 2n floats; stops when the residual estimate is <= max(rtol*|r0|, atol).
constexpr int kKrylovMaxDim = 64;
constexpr int kKrylovMaxParts = 64;
// A cycle that has not reduced the residual estimate below abort_ratio * |r0|
// after abort_after steps stops early with *stalled = 1.  With tg (a cycle
// starting from x = 0) the cycle also stops once the residual estimate meets
// tol * (anorm * |d|_inf + bnorm) / 4, |d| checked every 8 steps.
struct KrylovTarget {
  double tol, anorm, bnorm;
};
int fgmres_cycle(bool spd, int64_t n, const elem_t *A, int64_t lda,
                 const float *W, const int32_t *perm, elem_t *V, elem_t *Z,
                 float *F, int m, double rtol, double atol, int abort_after,
                 double abort_ratio, const KrylovTarget *tg, elem_t *d,
                 int *inner, double *res_est, int *stalled);
int getrf(int64_t n, elem_t *A, int64_t lda, int32_t *ipiv, int32_t *perm);
// Householder QR in place on R (m x n, m >= n); Q (m x m, may be null) gets
// the orthogonal factor (qr.cu).
int qr(int64_t m, int64_t n, elem_t *R, int64_t ldr, elem_t *Q, int64_t ldq);
int getrs(int64_t n, int64_t nrhs, const elem_t *LU, int64_t lda,
          const int32_t *perm, const elem_t *B, int64_t ldb, elem_t *X,
          int64_t ldx);
int potrf(int64_t n, elem_t *A, int64_t lda, int32_t *info);
int potrs(int64_t n, int64_t nrhs, const elem_t *L, int64_t lda, elem_t *B,
          int64_t ldb, const int32_t *info);
int trsm_left(bool lower, bool trans, bool unit, int64_t n, int64_t nrhs,
              const elem_t *T, int64_t ldt, elem_t *B, int64_t ldb,
              const int32_t *info);
int laswp(elem_t *A, int64_t lda, int64_t c0, int64_t c1, int64_t c2,
          int64_t c3, const int32_t *ipiv, int64_t k1, int64_t k2);
}  // namespace mgb
