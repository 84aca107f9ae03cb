/*
 * mat.h -- drop-in header for libmat's dense-solve hot path, GB300 build.
 *
 * Same types, macros, names and signatures as libmat's mat.h for the part of
 * its API this library implements.  Link the object code with
 *   -lmatgb_f32   (default element type float)
 *   -lmatgb_f64   (when compiled with -DMAT_DOUBLE_PRECISION)
 * The hot-path functions (mat_mul, mat_gemm, mat_syrk, mat_plu, mat_chol,
 * mat_solve*, ...) run on one GB300 (sm_103a) through hand-written CUDA
 * kernels; there is no CPU path for them.  Construction/accessor helpers are
 * plain host code (they manage host memory, as the reference's do).
 *
 * Differences a caller may notice (each is deliberate):
 *   - MATDEF/MAT_IMPLEMENTATION are accepted but have no effect: the
 *     implementation lives in the shared library, so a translation unit that
 *     does "#define MATDEF static inline / #define MAT_IMPLEMENTATION" (as the
 *     reference's own tests do) still compiles unchanged and links against it.
 *   - MAT_MALLOC/MAT_CALLOC/MAT_FREE are fixed to the C library's allocator
 *     when the library is built; overriding them in user code changes nothing.
 *   - Floating-point results differ from the reference's CPU build by rounding
 *     (different operation order on the GPU); pivot choices are the same on
 *     tie-free inputs.
 */
#ifndef MAT_H_
#define MAT_H_

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#define MAT_COLUMN_MAJOR
#define MAT_ARCH "GB300"

#ifndef MATDEF
#define MATDEF
#endif

/* Declarations always have external linkage, whatever the caller set MATDEF
 * to (mat.h:45-47 makes MATDEF the linkage of the reference's definitions). */
#define MATGB_API

#ifndef MAT_MALLOC
#define MAT_MALLOC(sz) malloc(sz)
#endif
#ifndef MAT_CALLOC
#define MAT_CALLOC(n, sz) calloc(n, sz)
#endif
#ifndef MAT_FREE
#define MAT_FREE(p) free(p)
#endif
#ifndef MAT_FREE_MAT
#define MAT_FREE_MAT(m)                                                        \
  do {                                                                         \
    MAT_FREE((m)->data);                                                       \
    MAT_FREE(m);                                                               \
  } while (0)
#endif
#ifndef MAT_FREE_PERM
#define MAT_FREE_PERM(p)                                                       \
  do {                                                                         \
    MAT_FREE((p)->data);                                                       \
    MAT_FREE(p);                                                               \
  } while (0)
#endif

/* BLAS-style transpose flags (mat.h:116-120). */
typedef enum { MAT_NO_TRANS = 0, MAT_TRANS = 1 } mat_trans_t;

/* Element type (mat.h:165-181). */
#ifdef MAT_DOUBLE_PRECISION
typedef double mat_elem_t;
#ifndef MAT_DEFAULT_EPSILON
#define MAT_DEFAULT_EPSILON 1e-9
#endif
#define MAT_FABS fabs
#define MAT_SQRT sqrt
#define MAT_HUGE_VAL HUGE_VAL
#else
typedef float mat_elem_t;
#ifndef MAT_DEFAULT_EPSILON
#define MAT_DEFAULT_EPSILON 1e-6f
#endif
#define MAT_FABS fabsf
#define MAT_SQRT sqrtf
#define MAT_HUGE_VAL HUGE_VALF
#endif

/* Logging (mat.h:294-325). */
#ifndef MAT_LOG_LEVEL
#define MAT_LOG_LEVEL 0
#endif
#if MAT_LOG_LEVEL > 0
#include <stdio.h>
#ifndef MAT_LOG_OUTPUT_ERR
#define MAT_LOG_OUTPUT_ERR(msg) fprintf(stderr, "%s\n", msg)
#endif
#ifndef MAT_LOG_OUTPUT
#define MAT_LOG_OUTPUT(msg) fprintf(stdout, "%s\n", msg)
#endif
#endif
#if MAT_LOG_LEVEL >= 1
#define MAT_LOG_ERROR(msg) MAT_LOG_OUTPUT_ERR("[ERROR] " msg)
#else
#define MAT_LOG_ERROR(msg)
#endif
#if MAT_LOG_LEVEL >= 2
#define MAT_LOG_WARN(msg) MAT_LOG_OUTPUT("[WARN] " msg)
#else
#define MAT_LOG_WARN(msg)
#endif
#if MAT_LOG_LEVEL >= 3
#define MAT_LOG_INFO(msg) MAT_LOG_OUTPUT("[INFO] " msg)
#else
#define MAT_LOG_INFO(msg)
#endif

/* Assertions (mat.h:328-357). */
#ifndef MAT_ASSERT
#include <assert.h>
#define MAT_ASSERT(x) assert(x)
#endif
#ifndef MAT_ASSERT_MAT
#define MAT_ASSERT_MAT(m)                                                      \
  do {                                                                         \
    MAT_ASSERT((m) != NULL);                                                   \
    MAT_ASSERT((m)->data != NULL);                                             \
    MAT_ASSERT((m)->rows > 0 && (m)->cols > 0);                                \
  } while (0)
#endif
#ifndef MAT_ASSERT_DIM
#define MAT_ASSERT_DIM(rows, cols)                                             \
  do {                                                                         \
    MAT_ASSERT((rows) > 0);                                                    \
    MAT_ASSERT((cols) > 0);                                                    \
  } while (0)
#endif
#ifndef MAT_ASSERT_SQUARE
#define MAT_ASSERT_SQUARE(m)                                                   \
  do {                                                                         \
    MAT_ASSERT_MAT(m);                                                         \
    MAT_ASSERT((m)->rows == (m)->cols);                                        \
  } while (0)
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Core types (mat.h:364-393): column-major, leading dimension = rows. */
typedef struct {
  size_t rows;
  size_t cols;
  mat_elem_t *data;
} Mat;

typedef struct {
  size_t x;
  size_t y;
} MatSize;

typedef Mat Vec;

typedef struct {
  size_t *data;
  size_t size;
} Perm;

#define MAT_IDX(m, i, j) ((j) * (m)->rows + (i))
#define MAT_AT(m, i, j) ((m)->data[MAT_IDX(m, i, j)])
#define MAT_SET(m, i, j, v) ((m)->data[MAT_IDX(m, i, j)] = (v))

/* ---- Construction & memory (host helpers; mat.h:398-456) ---------------- */
MATGB_API Mat *mat_empty(size_t rows, size_t cols);               /* mat.h:398 */
MATGB_API Mat *mat_mat(size_t rows, size_t cols);                 /* mat.h:401 */
MATGB_API Mat *mat_from(size_t rows, size_t cols,
                        const mat_elem_t *values);                /* mat.h:404 */
MATGB_API void mat_init(Mat *out, const mat_elem_t *values);      /* mat.h:407 */
MATGB_API void mat_free_mat(Mat *m);                              /* mat.h:410 */
MATGB_API Mat *mat_zeros(size_t rows, size_t cols);               /* mat.h:413 */
MATGB_API Mat *mat_ones(size_t rows, size_t cols);                /* mat.h:416 */
MATGB_API void mat_fill(Mat *out, mat_elem_t value);              /* mat.h:419 */
MATGB_API void mat_eye(Mat *out);                                 /* mat.h:422 */
MATGB_API Mat *mat_reye(size_t dim);                              /* mat.h:425 */
MATGB_API Vec *mat_vec(size_t dim);                               /* mat.h:428 */
MATGB_API Vec *mat_row_vec(size_t dim);                           /* mat.h:431 */
MATGB_API Vec *mat_vec_from(size_t dim, const mat_elem_t *values);/* mat.h:434 */
MATGB_API Perm *mat_perm(size_t n);                               /* mat.h:437 */
MATGB_API void mat_free_perm(Perm *p);                            /* mat.h:440 */
MATGB_API void mat_perm_identity(Perm *p);                        /* mat.h:443 */
MATGB_API Mat *mat_perm_mat(const Perm *p);                       /* mat.h:446 */
MATGB_API Mat *mat_copy(const Mat *m);                            /* mat.h:450 */
MATGB_API void mat_deep_copy(Mat *out, const Mat *src);           /* mat.h:453 */
MATGB_API Mat *mat_rdeep_copy(const Mat *m);                      /* mat.h:456 */

/* ---- Accessors & info (host helpers; mat.h:458-478) --------------------- */
MATGB_API mat_elem_t mat_at(const Mat *mat, size_t row, size_t col); /* :461 */
MATGB_API void mat_set_at(Mat *m, size_t row, size_t col,
                          mat_elem_t value);                      /* mat.h:464 */
MATGB_API MatSize mat_size(const Mat *m);                         /* mat.h:467 */
MATGB_API void mat_print(const Mat *m);                           /* mat.h:470 */
MATGB_API bool mat_equals(const Mat *a, const Mat *b);            /* mat.h:475 */
MATGB_API bool mat_equals_tol(const Mat *a, const Mat *b,
                              mat_elem_t epsilon);                /* mat.h:478 */
/* Transpose into a new matrix (host helper used by callers to form L^T). */
MATGB_API Mat *mat_rt(const Mat *m);                              /* mat.h:636 */

/* ---- Products (GPU; mat.h:564-567) -------------------------------------- */
/* out = a * b.  Replaces mat_mul, mat.h:564 (impl 1842-1850). */
MATGB_API void mat_mul(Mat *out, const Mat *a, const Mat *b);
/* Return a * b in a new matrix.  Replaces mat_rmul, mat.h:567 (1852-1862). */
MATGB_API Mat *mat_rmul(const Mat *a, const Mat *b);

/* ---- BLAS-2/3 (GPU; mat.h:596-625) -------------------------------------- */
/* y = alpha*A*x + beta*y.  Replaces mat_gemv, mat.h:597 (2137-2146). */
MATGB_API void mat_gemv(Vec *y, mat_elem_t alpha, const Mat *A, const Vec *x,
                        mat_elem_t beta);
/* y = alpha*A^T*x + beta*y: y[j] = beta*y[j] + alpha*dot(A[:,j], x), y read
 * even when beta = 0.  Replaces mat_gemv_t, mat.h:601 (2224-2248). */
MATGB_API void mat_gemv_t(Vec *y, mat_elem_t alpha, const Mat *A, const Vec *x,
                          mat_elem_t beta);
/* y += alpha*x, each product rounded before the sum: bit-identical to the
 * reference's scalar loop.  Replaces mat_axpy, mat.h:594 (2009-2015). */
MATGB_API void mat_axpy(Vec *y, mat_elem_t alpha, const Vec *x);
/* C = alpha*A*B + beta*C.  Replaces mat_gemm, mat.h:612 (2787-2796).  beta==0
 * does not read C (BLAS convention; the reference's NEON scal does the same,
 * its scalar path multiplies C by 0). */
MATGB_API void mat_gemm(Mat *C, mat_elem_t alpha, const Mat *A, const Mat *B,
                        mat_elem_t beta);
/* C = alpha*A*A^T + beta*C on the 'L' or 'U' triangle only; the other
 * triangle is left untouched.  Replaces mat_syrk, mat.h:617 (5670-5679). */
MATGB_API void mat_syrk(Mat *C, const Mat *A, mat_elem_t alpha,
                        mat_elem_t beta, char uplo);
/* C = alpha*A^T*A + beta*C on one triangle.  Replaces mat_syrk_t, mat.h:622
 * (5727-5735). */
MATGB_API void mat_syrk_t(Mat *C, const Mat *A, mat_elem_t alpha,
                          mat_elem_t beta, char uplo);

/* ---- Factorisations (GPU; mat.h:773-780) -------------------------------- */
/* P*A = L*U, partial pivoting.  L unit lower, U upper, both n x n and fully
 * written; p->data[i] = source row of row i.  Returns the number of row swaps.
 * A pivot with |value| < MAT_DEFAULT_EPSILON is swapped in but not divided by
 * (mat.h:4235-4236).  Replaces mat_plu, mat.h:776 (4436-4474). */
MATGB_API int mat_plu(const Mat *A, Mat *L, Mat *U, Perm *p);
/* P*A*Q = L*U, full pivoting: at step k the first entry (row-major from
 * (k,k)) of largest |value| in the trailing block is swapped into (k,k) --
 * rows first, then columns; a step whose largest |value| is below
 * MAT_DEFAULT_EPSILON is skipped.  L unit lower, U upper, both n x n;
 * p->data[i] / q->data[i] = source row / column of row / column i.
 * Returns the number of row plus column swaps; results are bit-identical to
 * the reference's scalar elimination.  Replaces mat_lu, mat.h:771
 * (4476-4574). */
MATGB_API int mat_lu(const Mat *A, Mat *L, Mat *U, Perm *p, Perm *q);
/* A = L*L^T from the lower triangle of A.  Returns 0, or -1 when a diagonal
 * is <= 0 (L then holds a partial factor).  Replaces mat_chol, mat.h:780
 * (6062-6092). */
MATGB_API int mat_chol(const Mat *A, Mat *L);
/* det(A) = (-1)^swaps * prod(diag U) from the GPU PLU.  Replaces mat_det,
 * mat.h:734 (6227-6249). */
MATGB_API mat_elem_t mat_det(const Mat *A);
/* A^{-1} via the GPU PLU and a multi-right-hand-side triangular solve.
 * Replaces mat_inv, mat.h:789 (6166-6225). */
MATGB_API void mat_inv(Mat *out, const Mat *A);

/* A (m x n, m >= n) = Q (m x m) * R (m x n) by Householder reflections with
 * the reference's reflector (beta = -sign(a_jj) |x|, v[0] = 1, no reflection
 * when |x| < MAT_DEFAULT_EPSILON), blocked in the WY form; R's entries below
 * the diagonal are the reflections' rounding residue, as in the reference.
 * Replaces mat_qr, mat.h:744 (3907-4064). */
MATGB_API void mat_qr(const Mat *A, Mat *Q, Mat *R);
/* The R factor alone (no Q accumulation).  Replaces mat_qr_r, mat.h:749
 * (4066-4192). */
MATGB_API void mat_qr_r(const Mat *A, Mat *R);

/* ---- Solvers (GPU; mat.h:821-838) --------------------------------------- */
/* Ax = b by PLU; only column 0 of b is read, as in the reference.  Replaces
 * mat_solve, mat.h:823 (4807-4837). */
MATGB_API void mat_solve(Vec *x, const Mat *A, const Vec *b);
/* Ax = b for SPD A by Cholesky; returns 0 or -1 (not positive definite, x
 * untouched).  Replaces mat_solve_spd, mat.h:828 (4839-4871). */
MATGB_API int mat_solve_spd(Vec *x, const Mat *A, const Vec *b);
/* Lx = b (non-unit lower).  Replaces mat_solve_tril, mat.h:832 (4626-4634). */
MATGB_API void mat_solve_tril(Vec *x, const Mat *L, const Vec *b);
/* Lx = b (unit lower).  Replaces mat_solve_tril_unit, mat.h:834 (4679-4687). */
MATGB_API void mat_solve_tril_unit(Vec *x, const Mat *L, const Vec *b);
/* Ux = b (upper).  Replaces mat_solve_triu, mat.h:836 (4738-4746). */
MATGB_API void mat_solve_triu(Vec *x, const Mat *U, const Vec *b);
/* L^T x = b using L directly.  Replaces mat_solve_trilt, mat.h:838
 * (4792-4803). */
MATGB_API void mat_solve_trilt(Vec *x, const Mat *L, const Vec *b);

#ifdef __cplusplus
}
#endif

/* A translation unit that defines MAT_IMPLEMENTATION gets the standard
 * headers the reference's implementation section includes (mat.h:858-862),
 * as code written against the reference may rely on them. */
#ifdef MAT_IMPLEMENTATION
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#endif

#endif /* MAT_H_ */
