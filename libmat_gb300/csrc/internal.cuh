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

// Record an error; returns `code`.  Never aborts (callers decide).
int set_error(int code, const char *fmt, ...);
// Record a CUDA failure with its call site.
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);
// For the void mat_* entry points: report and abort unless disabled.
void fail_void(const char *where);

// Host-side launch accounting + launch-error check.
int launched(const char *name);

// Optional per-kernel timing (matgb_ktime_enable): a scope records CUDA events
// on the library stream around one launch and tags it with the launch's
// algorithmic FLOPs and bytes.  Costs nothing when disabled.
struct KtScope {
  int idx;
  KtScope(const char *name, double flops, double bytes);
  ~KtScope();
};

// Grow-only device buffers keyed by slot, reused across calls (the device
// counterpart of the reference's scratch arena, mat.h:865-895).
enum WsSlot {
  WS_A = 0, WS_B, WS_C, WS_X, WS_L, WS_U, WS_PIV, WS_INFO,
  WS_T0, WS_T1, WS_T2, WS_T3, WS_NSLOTS
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
int getrf(int64_t n, elem_t *A, int64_t lda, int32_t *ipiv, int32_t *perm);
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
