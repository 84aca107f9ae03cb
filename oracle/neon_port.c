/*
 * CPU BASELINE ONLY (test infrastructure: bench.py's CPU legs and tests/).
 * Nothing in the shipped library loads this file.
 *
 * A restatement of the reference's mat_solve on its ARM NEON path, double
 * precision, for timing the reference's CPU algorithm on the GPU host's
 * Grace cores (the reference's source is not present there, so its own
 * build cannot run on that host):
 *   - mat__plu_blocked_ (mat.h:4201-4289): 24-column panels with partial
 *     pivoting (first index of max |a|, mat__iamax mat.h:1247-1262), the
 *     delayed row swaps, the unit-lower TRSM for U12, and the trailing update
 *     A22 -= L21 U12 by
 *   - mat__gemm_strided_neon_ (mat.h:2470-2716): C scaled by beta, K blocks
 *     of KC = 256, A packed in panels of MR = 8 rows, B in panels of NR = 4
 *     columns (double), an 8 x 4 micro-kernel holding the tile in 16
 *     two-lane accumulators updated by lane-broadcast FMAs, remainder rows and
 *     columns by scalar loops;
 *   - the triangular solves of mat_solve (mat.h:4807-4837) in column order.
 * On an aarch64 host the micro-kernel uses arm_neon.h (MAT_ARCH "NEON");
 * elsewhere the same packed loops run in plain C ("SCALAR-packed") so the
 * file builds and can be checked against the oracle on any host.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#if defined(__aarch64__)
#include <arm_neon.h>
#define NP_NEON 1
#endif

typedef double T;
#define NP_EPS 1e-9 /* MAT_DEFAULT_EPSILON in double (mat.h:168-176) */
#define NP_NB 24    /* MAT_PLU_BLOCK_SIZE (mat.h:4196) */
#define NP_KC 256
#define NP_MR 8
#define NP_NR 4

const char *np_arch(void) {
#ifdef NP_NEON
  return "NEON";
#else
  return "SCALAR-packed";
#endif
}

/* C (M x N, ldc) = beta C + alpha op(A) op(B), column-major, no transposes
 * needed here (the LU update is NN). */
static void gemm_nn(T *C, size_t ldc, T alpha, const T *A, size_t lda,
                    const T *B, size_t ldb, size_t M, size_t K, size_t N,
                    T beta, T *pa_buf, T *pb_buf) {
  for (size_t j = 0; j < N; j++)
    for (size_t i = 0; i < M; i++) C[j * ldc + i] *= beta;
  const size_t M8 = M / NP_MR * NP_MR, N4 = N / NP_NR * NP_NR;
  const size_t npa = M8 / NP_MR;
  for (size_t k0 = 0; k0 < K; k0 += NP_KC) {
    const size_t kc = k0 + NP_KC <= K ? NP_KC : K - k0;
    for (size_t p = 0; p < npa; p++) {
      T *pa = pa_buf + p * NP_KC * NP_MR;
      for (size_t kk = 0; kk < kc; kk++)
        for (size_t ii = 0; ii < NP_MR; ii++)
          pa[kk * NP_MR + ii] = A[(k0 + kk) * lda + p * NP_MR + ii];
    }
    for (size_t j = 0; j < N4; j += NP_NR) {
      for (size_t kk = 0; kk < kc; kk++)
        for (size_t jj = 0; jj < NP_NR; jj++)
          pb_buf[kk * NP_NR + jj] = B[(j + jj) * ldb + k0 + kk];
      for (size_t p = 0; p < npa; p++) {
        const T *pa = pa_buf + p * NP_KC * NP_MR;
        T *cp = C + j * ldc + p * NP_MR;
#ifdef NP_NEON
        float64x2_t c[NP_NR][4];
        for (int jj = 0; jj < NP_NR; jj++)
          for (int r = 0; r < 4; r++) c[jj][r] = vdupq_n_f64(0.0);
        for (size_t kk = 0; kk < kc; kk++) {
          const float64x2_t a0 = vld1q_f64(pa + kk * NP_MR);
          const float64x2_t a1 = vld1q_f64(pa + kk * NP_MR + 2);
          const float64x2_t a2 = vld1q_f64(pa + kk * NP_MR + 4);
          const float64x2_t a3 = vld1q_f64(pa + kk * NP_MR + 6);
          const float64x2_t b01 = vld1q_f64(pb_buf + kk * NP_NR);
          const float64x2_t b23 = vld1q_f64(pb_buf + kk * NP_NR + 2);
          c[0][0] = vfmaq_laneq_f64(c[0][0], a0, b01, 0);
          c[0][1] = vfmaq_laneq_f64(c[0][1], a1, b01, 0);
          c[0][2] = vfmaq_laneq_f64(c[0][2], a2, b01, 0);
          c[0][3] = vfmaq_laneq_f64(c[0][3], a3, b01, 0);
          c[1][0] = vfmaq_laneq_f64(c[1][0], a0, b01, 1);
          c[1][1] = vfmaq_laneq_f64(c[1][1], a1, b01, 1);
          c[1][2] = vfmaq_laneq_f64(c[1][2], a2, b01, 1);
          c[1][3] = vfmaq_laneq_f64(c[1][3], a3, b01, 1);
          c[2][0] = vfmaq_laneq_f64(c[2][0], a0, b23, 0);
          c[2][1] = vfmaq_laneq_f64(c[2][1], a1, b23, 0);
          c[2][2] = vfmaq_laneq_f64(c[2][2], a2, b23, 0);
          c[2][3] = vfmaq_laneq_f64(c[2][3], a3, b23, 0);
          c[3][0] = vfmaq_laneq_f64(c[3][0], a0, b23, 1);
          c[3][1] = vfmaq_laneq_f64(c[3][1], a1, b23, 1);
          c[3][2] = vfmaq_laneq_f64(c[3][2], a2, b23, 1);
          c[3][3] = vfmaq_laneq_f64(c[3][3], a3, b23, 1);
        }
        const float64x2_t va = vdupq_n_f64(alpha);
        for (int jj = 0; jj < NP_NR; jj++)
          for (int r = 0; r < 4; r++) {
            T *dst = cp + jj * ldc + 2 * r;
            vst1q_f64(dst, vfmaq_f64(vld1q_f64(dst), va, c[jj][r]));
          }
#else
        T c[NP_NR][NP_MR];
        memset(c, 0, sizeof c);
        for (size_t kk = 0; kk < kc; kk++)
          for (int jj = 0; jj < NP_NR; jj++) {
            const T bv = pb_buf[kk * NP_NR + jj];
            for (int ii = 0; ii < NP_MR; ii++) c[jj][ii] += pa[kk * NP_MR + ii] * bv;
          }
        for (int jj = 0; jj < NP_NR; jj++)
          for (int ii = 0; ii < NP_MR; ii++) cp[jj * ldc + ii] += alpha * c[jj][ii];
#endif
      }
    }
    /* remainder rows (M8..M) of the N4 columns, and remainder columns */
    for (size_t j = 0; j < N; j++) {
      const size_t i0 = j < N4 ? M8 : 0;
      for (size_t kk = 0; kk < kc; kk++) {
        const T bv = alpha * B[j * ldb + k0 + kk];
        const T *acol = A + (k0 + kk) * lda;
        T *ccol = C + j * ldc;
        for (size_t i = i0; i < M; i++) ccol[i] += acol[i] * bv;
      }
    }
  }
}

/* first index of max |x| (mat__iamax: NaN at the start wins, later NaN
 * never compares greater) */
static size_t iamax(const T *x, size_t n) {
  size_t best = 0;
  T bv = fabs(x[0]);
  for (size_t i = 1; i < n; i++) {
    const T v = fabs(x[i]);
    if (v > bv) {
      bv = v;
      best = i;
    }
  }
  return best;
}

/* In-place blocked PLU of the n x n column-major M; p[i] = source row of row
 * i.  Returns the swap count. */
int np_plu_inplace(T *M, size_t n, size_t *p) {
  for (size_t i = 0; i < n; i++) p[i] = i;
  int swaps = 0;
  size_t piv[NP_NB];
  T *pa = (T *)malloc(((n + NP_MR) / NP_MR + 1) * NP_KC * NP_MR * sizeof(T));
  T *pb = (T *)malloc(NP_KC * NP_NR * sizeof(T));
  for (size_t kb = 0; kb < n; kb += NP_NB) {
    const size_t ke = kb + NP_NB < n ? kb + NP_NB : n;
    for (size_t k = kb; k < ke && k < n - 1; k++) {
      T *ck = M + k * n;
      const size_t pr = k + iamax(ck + k, n - k);
      piv[k - kb] = pr;
      if (pr != k) {
        for (size_t j = 0; j < ke; j++) {
          T t = M[j * n + k];
          M[j * n + k] = M[j * n + pr];
          M[j * n + pr] = t;
        }
        size_t t = p[k];
        p[k] = p[pr];
        p[pr] = t;
        swaps++;
      }
      if (fabs(ck[k]) < NP_EPS) continue;
      const T inv = 1.0 / ck[k];
      for (size_t i = k + 1; i < n; i++) ck[i] *= inv;
      for (size_t j = k + 1; j < ke; j++) {
        T *cj = M + j * n;
        const T f = -cj[k];
        for (size_t i = k + 1; i < n; i++) cj[i] += f * ck[i];
      }
    }
    if (ke < n) {
      for (size_t k = kb; k < ke && k < n - 1; k++) {
        const size_t pr = piv[k - kb];
        if (pr != k)
          for (size_t j = ke; j < n; j++) {
            T t = M[j * n + k];
            M[j * n + k] = M[j * n + pr];
            M[j * n + pr] = t;
          }
      }
      for (size_t k = kb; k < ke; k++) {
        const T *ck = M + k * n;
        for (size_t j = ke; j < n; j++) {
          T *cj = M + j * n;
          const T f = -cj[k];
          for (size_t i = k + 1; i < ke; i++) cj[i] += f * ck[i];
        }
      }
      gemm_nn(M + ke * n + ke, n, -1.0, M + kb * n + ke, n, M + ke * n + kb, n,
              n - ke, ke - kb, n - ke, 1.0, pa, pb);
    }
  }
  free(pa);
  free(pb);
  return swaps;
}

/* x = A^{-1} b: PLU, b[p], unit-lower then upper solves (column order) */
void np_solve(T *x, const T *A, const T *b, size_t n) {
  T *M = (T *)malloc(n * n * sizeof(T));
  size_t *p = (size_t *)malloc(n * sizeof(size_t));
  memcpy(M, A, n * n * sizeof(T));
  np_plu_inplace(M, n, p);
  for (size_t i = 0; i < n; i++) x[i] = b[p[i]];
  for (size_t j = 0; j < n; j++) {
    const T xj = x[j];
    const T *cj = M + j * n;
    for (size_t i = j + 1; i < n; i++) x[i] -= cj[i] * xj;
  }
  for (size_t jj = n; jj-- > 0;) {
    const T *cj = M + jj * n;
    x[jj] /= cj[jj];
    const T xj = x[jj];
    for (size_t i = 0; i < jj; i++) x[i] -= cj[i] * xj;
  }
  free(M);
  free(p);
}
