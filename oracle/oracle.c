/*
 * CPU oracle for the dense-solve hot path of libmat (TEST INFRASTRUCTURE).
 *
 * This file restates, in plain C, the algorithm that libmat's scalar build
 * runs for mat_gemm / mat_plu / mat_chol / mat_syrk / mat_solve_tri* /
 * mat_solve / mat_solve_spd.  It exists only as a checker: the test-suite and
 * bench.py's CPU-baseline leg call it through ctypes to compare and time.
 * Nothing in the shipped library links, loads or calls it.
 *
 * Every routine cites the reference file:line it follows (mat.h of
 * alvgaona/libmat).  The operation order matches the reference's scalar path
 * (the one its x86 build takes), and the file is compiled with
 * -ffp-contract=off so that products and sums round separately, as they do in
 * the reference's x86 build.  It is pinned bit-for-bit against the reference
 * itself (compiled from its own header into oracle/_ref) by the CPU tests.
 *
 * Element type: float by default, double with -DORC_DOUBLE (the reference's
 * MAT_DOUBLE_PRECISION).  Storage is column-major, leading dimension = rows.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef ORC_DOUBLE
typedef double T;
#define ORC_EPS 1e-9 /* MAT_DEFAULT_EPSILON, mat.h:168 */
#define ORC_FABS fabs
#define ORC_SQRT sqrt
#define ORC_ONE_F 1.0 /* (1.0f promoted to double in the reference) */
#else
typedef float T;
#define ORC_EPS 1e-6f /* MAT_DEFAULT_EPSILON, mat.h:176 */
#define ORC_FABS fabsf
#define ORC_SQRT sqrtf
#define ORC_ONE_F 1.0f
#endif

#define AT(p, ld, i, j) ((p)[(size_t)(j) * (ld) + (i)])

int orc_elem_size(void) { return (int)sizeof(T); }

/* y *= alpha -- mat__scal_scalar, mat.h:960-964 */
static void scal(T *y, T alpha, size_t n) {
  for (size_t i = 0; i < n; i++) y[i] *= alpha;
}

/* y += alpha * x -- mat__axpy_scalar, mat.h:908-913 */
static void axpy(T *y, T alpha, const T *x, size_t n) {
  for (size_t i = 0; i < n; i++) y[i] += alpha * x[i];
}

/* dot product, accumulated from 0 in index order -- mat__dot_scalar,
 * mat.h:1003-1010 */
static T dot(const T *a, const T *b, size_t n) {
  T r = 0;
  for (size_t i = 0; i < n; i++) r += a[i] * b[i];
  return r;
}

/* First index of max |x| -- mat__amax_scalar + mat__iamax, mat.h:1196-1262.
 * amax folds with '>' starting from |x[0]| (so a NaN in x[0] poisons it and a
 * later NaN is ignored); the index is the first i with |x[i]| == max, or 0
 * when nothing compares equal (the NaN case). */
size_t orc_iamax(const T *x, size_t n) {
  if (n == 0) return 0;
  T m = ORC_FABS(x[0]);
  for (size_t i = 1; i < n; i++) {
    T v = ORC_FABS(x[i]);
    if (v > m) m = v;
  }
  for (size_t i = 0; i < n; i++)
    if (ORC_FABS(x[i]) == m) return i;
  return 0;
}

/* C = alpha*A*B + beta*C, A m x k, B k x n -- mat__gemm_scalar,
 * mat.h:2762-2785: scale C by beta, then ikj with aik = alpha*A[i,k]. */
void orc_gemm(size_t m, size_t k, size_t n, T alpha, const T *A, const T *B,
              T beta, T *C) {
  scal(C, beta, m * n);
  for (size_t i = 0; i < m; i++)
    for (size_t p = 0; p < k; p++) {
      T aik = alpha * AT(A, m, i, p);
      for (size_t j = 0; j < n; j++)
        AT(C, m, i, j) = AT(C, m, i, j) + aik * AT(B, k, p, j);
    }
}

/* Strided GEMM used by the blocked LU -- mat__gemm_strided_ scalar fallback,
 * mat.h:2719-2741 (no-transpose operands only, which is all the LU uses). */
static void gemm_strided(T *C, size_t ldc, T alpha, const T *A, size_t lda,
                         const T *B, size_t ldb, size_t M, size_t K, size_t N,
                         T beta) {
  for (size_t j = 0; j < N; j++) scal(&C[j * ldc], beta, M);
  for (size_t j = 0; j < N; j++)
    for (size_t p = 0; p < K; p++) {
      T ab = alpha * B[j * ldb + p];
      for (size_t i = 0; i < M; i++) C[j * ldc + i] += A[p * lda + i] * ab;
    }
}

#define ORC_PLU_NB 24 /* MAT_PLU_BLOCK_SIZE, mat.h:4196 */

/* In-place blocked partial-pivot LU of the n x n column-major M with delayed
 * pivoting -- mat__plu_blocked_, mat.h:4201-4289.  perm (size n) must hold
 * the identity on entry; on return perm[i] is the source row of row i.
 * ipiv (optional, size n) receives the pivot row chosen at each step (k for
 * the last column, which the reference never searches).  Returns the swap
 * count. */
int orc_plu_inplace(T *M, size_t n, size_t *perm, size_t *ipiv) {
  int swaps = 0;
  size_t prow[ORC_PLU_NB];
  if (ipiv)
    for (size_t i = 0; i < n; i++) ipiv[i] = i;
  for (size_t kb = 0; kb < n; kb += ORC_PLU_NB) {
    size_t ke = kb + ORC_PLU_NB < n ? kb + ORC_PLU_NB : n;
    size_t bk = ke - kb;
    for (size_t k = kb; k < ke && k < n - 1; k++) {
      T *ck = &M[k * n];
      size_t p = k + orc_iamax(&ck[k], n - k);
      prow[k - kb] = p;
      if (ipiv) ipiv[k] = p;
      if (p != k) {
        for (size_t j = 0; j < ke; j++) {
          T *cj = &M[j * n];
          T t = cj[k];
          cj[k] = cj[p];
          cj[p] = t;
        }
        size_t t = perm[k];
        perm[k] = perm[p];
        perm[p] = t;
        swaps++;
      }
      if (ORC_FABS(ck[k]) < ORC_EPS) continue; /* pivot skip, mat.h:4235 */
      T inv = ORC_ONE_F / ck[k];
      scal(&ck[k + 1], inv, n - (k + 1));
      for (size_t j = k + 1; j < ke; j++) {
        T *cj = &M[j * n];
        axpy(&cj[k + 1], -cj[k], &ck[k + 1], n - (k + 1));
      }
    }
    if (ke < n) {
      for (size_t k = kb; k < ke && k < n - 1; k++) {
        size_t p = prow[k - kb];
        if (p != k)
          for (size_t j = ke; j < n; j++) {
            T *cj = &M[j * n];
            T t = cj[k];
            cj[k] = cj[p];
            cj[p] = t;
          }
      }
      for (size_t k = kb; k < ke; k++) {
        T *ck = &M[k * n];
        for (size_t j = ke; j < n; j++) {
          T *cj = &M[j * n];
          axpy(&cj[k + 1], -cj[k], &ck[k + 1], ke - (k + 1));
        }
      }
      gemm_strided(&M[ke * n + ke], n, (T)-1, &M[kb * n + ke], n,
                   &M[ke * n + kb], n, n - ke, bk, n - ke, (T)1);
    }
  }
  return swaps;
}

/* mat_plu, mat.h:4436-4474: copy A, factor, split into unit-lower L and
 * upper U (both n x n, fully written). */
int orc_plu(const T *A, size_t n, T *L, T *U, size_t *perm) {
  T *M = (T *)malloc(n * n * sizeof(T));
  memcpy(M, A, n * n * sizeof(T));
  for (size_t i = 0; i < n; i++) perm[i] = i;
  int swaps = orc_plu_inplace(M, n, perm, NULL);
  memset(L, 0, n * n * sizeof(T));
  memset(U, 0, n * n * sizeof(T));
  for (size_t j = 0; j < n; j++) {
    L[j * n + j] = 1;
    for (size_t i = j + 1; i < n; i++) L[j * n + i] = M[j * n + i];
    for (size_t i = 0; i <= j; i++) U[j * n + i] = M[j * n + i];
  }
  free(M);
  return swaps;
}

/* mat_lu, mat.h:4476-4574 (the scalar branch, 4502-4555): full pivoting.
 * Per step the pivot is the first entry, scanning rows i = k.. and within a
 * row columns j = k.., whose |a| is strictly larger than the best so far
 * (starting from a_kk); below MAT_DEFAULT_EPSILON the step is skipped.  Whole
 * rows then whole columns are exchanged (p, q record them), column k is
 * scaled by 1.0f / a_kk and the trailing block takes the rank-1 update.
 * L unit-lower and U upper as mat_lu writes them; returns the swap count. */
int orc_lu(const T *A, size_t n, T *L, T *U, size_t *p, size_t *q) {
  T *data = (T *)malloc(n * n * sizeof(T));
  memcpy(data, A, n * n * sizeof(T));
  for (size_t i = 0; i < n; i++) p[i] = q[i] = i;
  int swaps = 0;
  for (size_t k = 0; k + 1 < n; k++) {
    size_t pr = k, pc = k;
    T mx = ORC_FABS(data[k * n + k]);
    for (size_t i = k; i < n; i++)
      for (size_t j = k; j < n; j++) {
        const T v = ORC_FABS(data[j * n + i]);
        if (v > mx) {
          mx = v;
          pr = i;
          pc = j;
        }
      }
    if (mx < ORC_EPS) continue;
    if (pr != k) {
      for (size_t j = 0; j < n; j++) {
        const T t = data[j * n + k];
        data[j * n + k] = data[j * n + pr];
        data[j * n + pr] = t;
      }
      const size_t t = p[k];
      p[k] = p[pr];
      p[pr] = t;
      swaps++;
    }
    if (pc != k) {
      for (size_t i = 0; i < n; i++) {
        const T t = data[k * n + i];
        data[k * n + i] = data[pc * n + i];
        data[pc * n + i] = t;
      }
      const size_t t = q[k];
      q[k] = q[pc];
      q[pc] = t;
      swaps++;
    }
    const T inv = ORC_ONE_F / data[k * n + k];
    for (size_t i = k + 1; i < n; i++) {
      const T l = data[k * n + i] * inv;
      data[k * n + i] = l;
      for (size_t j = k + 1; j < n; j++) data[j * n + i] -= l * data[j * n + k];
    }
  }
  memset(L, 0, n * n * sizeof(T));
  memset(U, 0, n * n * sizeof(T));
  for (size_t j = 0; j < n; j++) {
    L[j * n + j] = 1;
    for (size_t i = j + 1; i < n; i++) L[j * n + i] = data[j * n + i];
    for (size_t i = 0; i <= j; i++) U[j * n + i] = data[j * n + i];
  }
  free(data);
  return swaps;
}

/* Lx = b, non-unit -- mat__solve_tril_scalar, mat.h:4584-4598 */
void orc_solve_tril(T *x, const T *L, const T *b, size_t n) {
  for (size_t i = 0; i < n; i++) {
    T d = 0;
    for (size_t j = 0; j < i; j++) d += AT(L, n, i, j) * x[j];
    x[i] = (b[i] - d) / AT(L, n, i, i);
  }
}

/* Lx = b, unit diagonal -- mat__solve_tril_unit_scalar, mat.h:4638-4652 */
void orc_solve_tril_unit(T *x, const T *L, const T *b, size_t n) {
  for (size_t i = 0; i < n; i++) {
    T d = 0;
    for (size_t j = 0; j < i; j++) d += AT(L, n, i, j) * x[j];
    x[i] = b[i] - d;
  }
}

/* Ux = b -- mat__solve_triu_scalar, mat.h:4722-4736 */
void orc_solve_triu(T *x, const T *U, const T *b, size_t n) {
  for (size_t i = n; i-- > 0;) {
    T s = b[i];
    for (size_t j = i + 1; j < n; j++) s -= AT(U, n, i, j) * x[j];
    x[i] = s / AT(U, n, i, i);
  }
}

/* L^T x = b with column dots -- mat__solve_trilt_scalar, mat.h:4766-4780 */
void orc_solve_trilt(T *x, const T *L, const T *b, size_t n) {
  for (size_t j = n; j-- > 0;) {
    const T *Lj = &L[j * n];
    T d = 0;
    for (size_t k = j + 1; k < n; k++) d += Lj[k] * x[k];
    x[j] = (b[j] - d) / Lj[j];
  }
}

/* mat_solve, mat.h:4807-4837: PLU, pb = b[p] (column 0 only), unit-lower
 * forward solve, upper back solve. */
void orc_solve(T *x, const T *A, const T *b, size_t n) {
  T *L = (T *)malloc(n * n * sizeof(T));
  T *U = (T *)malloc(n * n * sizeof(T));
  size_t *p = (size_t *)malloc(n * sizeof(size_t));
  T *pb = (T *)malloc(n * sizeof(T));
  T *z = (T *)malloc(n * sizeof(T));
  orc_plu(A, n, L, U, p);
  for (size_t i = 0; i < n; i++) pb[i] = b[p[i]];
  orc_solve_tril_unit(z, L, pb, n);
  orc_solve_triu(x, U, z, n);
  free(L);
  free(U);
  free(p);
  free(pb);
  free(z);
}

/* mat_chol, mat.h:6062-6092, scalar path mat__chol_scalar_generic_,
 * mat.h:6031-6060: copy the lower triangle, zero the upper, dot-form
 * column Cholesky.  Returns 0, or -1 at the first diagonal <= 0 (L then holds
 * the partial factor). */
int orc_chol(const T *A, size_t n, T *L) {
  for (size_t j = 0; j < n; j++) {
    for (size_t i = 0; i < j; i++) L[j * n + i] = 0;
    memcpy(&L[j * n + j], &A[j * n + j], (n - j) * sizeof(T));
  }
  for (size_t j = 0; j < n; j++) {
    T s = 0;
    for (size_t k = 0; k < j; k++) {
      T ljk = AT(L, n, j, k);
      s += ljk * ljk;
    }
    T diag = AT(L, n, j, j) - s;
    if (diag <= 0) return -1;
    T ljj = ORC_SQRT(diag);
    AT(L, n, j, j) = ljj;
    T inv = ORC_ONE_F / ljj;
    for (size_t i = j + 1; i < n; i++) {
      T d = 0;
      for (size_t k = 0; k < j; k++) d += AT(L, n, i, k) * AT(L, n, j, k);
      AT(L, n, i, j) = (AT(L, n, i, j) - d) * inv;
    }
  }
  return 0;
}

/* mat_solve_spd, mat.h:4839-4871: Cholesky, Ly = b, L^T x = y. */
int orc_solve_spd(T *x, const T *A, const T *b, size_t n) {
  T *L = (T *)malloc(n * n * sizeof(T));
  T *y = (T *)malloc(n * sizeof(T));
  int r = orc_chol(A, n, L);
  if (r == 0) {
    orc_solve_tril(y, L, b, n);
    orc_solve_trilt(x, L, y, n);
  }
  free(L);
  free(y);
  return r == 0 ? 0 : -1;
}

/* mat_syrk, scalar mat__syrk_scalar, mat.h:5641-5668: C (n x n) gets
 * beta*C + alpha*A*A^T on the requested triangle only; A is n x k. */
void orc_syrk(T *C, const T *A, size_t n, size_t k, T alpha, T beta,
              char uplo) {
  int lower = (uplo == 'L' || uplo == 'l');
  for (size_t i = 0; i < n; i++) {
    size_t j0 = lower ? 0 : i, j1 = lower ? i + 1 : n;
    for (size_t j = j0; j < j1; j++) {
      T s = 0;
      for (size_t p = 0; p < k; p++) s += AT(A, n, i, p) * AT(A, n, j, p);
      AT(C, n, i, j) = beta * AT(C, n, i, j) + alpha * s;
    }
  }
}

/* mat_syrk_t: C (n x n) gets beta*C + alpha*A^T*A on one triangle; A is
 * k x n -- mat__syrk_t_scalar, mat.h:5697-5725. */
void orc_syrk_t(T *C, const T *A, size_t n, size_t k, T alpha, T beta,
                char uplo) {
  int lower = (uplo == 'L' || uplo == 'l');
  for (size_t i = 0; i < n; i++) {
    size_t j0 = lower ? 0 : i, j1 = lower ? i + 1 : n;
    for (size_t j = j0; j < j1; j++) {
      T s = 0;
      for (size_t p = 0; p < k; p++) s += AT(A, k, p, i) * AT(A, k, p, j);
      AT(C, n, i, j) = beta * AT(C, n, i, j) + alpha * s;
    }
  }
}

/* y = alpha*A*x + beta*y, A m x n -- mat__gemv_scalar, mat.h:2121-2135 */
/* y[j] = beta*y[j] + alpha*dot(A[:,j], x) -- mat__gemv_t_scalar,
 * mat.h:2224-2237, the dot in index order as mat__dot_scalar (1003-1010) */
void orc_gemv_t(T *y, T alpha, const T *A, const T *x, T beta, size_t m,
                size_t n) {
  for (size_t j = 0; j < n; j++) {
    T d = 0;
    for (size_t i = 0; i < m; i++) d += A[j * m + i] * x[i];
    y[j] = beta * y[j] + alpha * d;
  }
}

/* Householder vector of x (n entries): v[0] = 1, H = I - tau v v^T maps x
 * to beta e1 with beta = -sign(x0) ||x||; tau = 0 and v = 0 when ||x|| is
 * below eps -- mat_householder, mat.h:3636-3718 (scalar branch). */
static T householder(T *v, T *tau, const T *x, size_t n) {
  if (n == 0) {
    *tau = 0;
    return 0;
  }
  T norm_sq = 0;
  for (size_t i = 0; i < n; i++) norm_sq += x[i] * x[i];
  const T norm_x = ORC_SQRT(norm_sq);
  if (norm_x < ORC_EPS) {
    *tau = 0;
    for (size_t i = 0; i < n; i++) v[i] = 0;
    return 0;
  }
  const T x0 = x[0];
  const T beta = (x0 >= 0) ? -norm_x : norm_x;
  const T v0 = x0 - beta;
  const T v0_inv = 1 / v0;
  v[0] = 1;
  for (size_t i = 1; i < n; i++) v[i] = x[i] * v0_inv;
  *tau = -v0 / beta;
  return beta;
}

/* A (m x n, m >= n) = Q (m x m) R (m x n) by Householder reflections, one
 * column at a time: the reference's unblocked path (n < 64), mat.h:
 * 4016-4060.  R's entries below the diagonal are what the reflections leave
 * there (not set to zero), as in the reference. */
void orc_qr(const T *A, size_t m, size_t n, T *Q, T *R) {
  memcpy(R, A, m * n * sizeof(T));
  memset(Q, 0, m * m * sizeof(T));
  for (size_t i = 0; i < m; i++) Q[i * m + i] = 1;
  T *x = (T *)malloc((m + 1) * sizeof(T));
  T *v = (T *)malloc((m + 1) * sizeof(T));
  T *u = (T *)malloc((m + 1) * sizeof(T));
  for (size_t j = 0; j < n; j++) {
    const size_t len = m - j;
    memcpy(x, &R[j * m + j], len * sizeof(T));
    T tau;
    (void)householder(v, &tau, x, len);
    if (tau == 0) continue;
    for (size_t k = j; k < n; k++) {
      T *Rk = &R[k * m + j];
      const T w = tau * dot(v, Rk, len);
      axpy(Rk, -w, v, len);
    }
    memset(u, 0, m * sizeof(T));
    for (size_t jj = 0; jj < len; jj++) axpy(u, v[jj], &Q[(j + jj) * m], m);
    for (size_t jj = 0; jj < len; jj++)
      axpy(&Q[(j + jj) * m], -tau * v[jj], u, m);
  }
  free(x);
  free(v);
  free(u);
}

/* y += alpha*x -- mat_axpy, mat.h:2009-2015 via mat__axpy_scalar (909-914) */
void orc_axpy(T *y, T alpha, const T *x, size_t n) { axpy(y, alpha, x, n); }

void orc_gemv(T *y, T alpha, const T *A, const T *x, T beta, size_t m,
              size_t n) {
  scal(y, beta, m);
  for (size_t j = 0; j < n; j++) axpy(y, alpha * x[j], &A[j * m], m);
}
