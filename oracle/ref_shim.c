/*
 * Raw-pointer wrappers around libmat's own mat.h (TEST INFRASTRUCTURE).
 *
 * Compiled by oracle/Makefile directly from the reference header where it
 * lies (-I<reference dir>); nothing of the reference is copied here.  The
 * resulting oracle/_ref/libref_{f32,f64}.so are used to pin the C restatement
 * in oracle.c and to generate tests/golden fixtures.  Same signatures as
 * oracle.c with a ref_ prefix.
 *
 * MATDEF must be "static inline": an extern build of the reference does not
 * link on non-NEON hosts (mat_norm_fro_fast dispatches to a scalar symbol that
 * does not exist, mat.h:3534-3538).
 */
#define MATDEF static inline
#define MAT_IMPLEMENTATION
#include "mat.h"

#include <string.h>

static Mat wrap(size_t r, size_t c, const mat_elem_t *p) {
  Mat m;
  m.rows = r;
  m.cols = c;
  m.data = (mat_elem_t *)p;
  return m;
}

const char *ref_arch(void) { return MAT_ARCH; }
int ref_elem_size(void) { return (int)sizeof(mat_elem_t); }

void ref_gemm(size_t m, size_t k, size_t n, mat_elem_t alpha,
              const mat_elem_t *A, const mat_elem_t *B, mat_elem_t beta,
              mat_elem_t *C) {
  Mat a = wrap(m, k, A), b = wrap(k, n, B), c = wrap(m, n, C);
  mat_gemm(&c, alpha, &a, &b, beta);
}

void ref_mul(size_t m, size_t k, size_t n, const mat_elem_t *A,
             const mat_elem_t *B, mat_elem_t *C) {
  Mat a = wrap(m, k, A), b = wrap(k, n, B), c = wrap(m, n, C);
  mat_mul(&c, &a, &b);
}

int ref_plu(const mat_elem_t *A, size_t n, mat_elem_t *L, mat_elem_t *U,
            size_t *perm) {
  Mat a = wrap(n, n, A), l = wrap(n, n, L), u = wrap(n, n, U);
  Perm p;
  p.data = perm;
  p.size = n;
  return mat_plu(&a, &l, &u, &p);
}

int ref_lu(const mat_elem_t *A, size_t n, mat_elem_t *L, mat_elem_t *U,
           size_t *p, size_t *q) {
  Mat a = wrap(n, n, A), l = wrap(n, n, L), u = wrap(n, n, U);
  Perm pp, qq;
  pp.data = p;
  pp.size = n;
  qq.data = q;
  qq.size = n;
  return mat_lu(&a, &l, &u, &pp, &qq);
}

int ref_chol(const mat_elem_t *A, size_t n, mat_elem_t *L) {
  Mat a = wrap(n, n, A), l = wrap(n, n, L);
  return mat_chol(&a, &l);
}

void ref_syrk(mat_elem_t *C, const mat_elem_t *A, size_t n, size_t k,
              mat_elem_t alpha, mat_elem_t beta, char uplo) {
  Mat c = wrap(n, n, C), a = wrap(n, k, A);
  mat_syrk(&c, &a, alpha, beta, uplo);
}

void ref_syrk_t(mat_elem_t *C, const mat_elem_t *A, size_t n, size_t k,
                mat_elem_t alpha, mat_elem_t beta, char uplo) {
  Mat c = wrap(n, n, C), a = wrap(k, n, A);
  mat_syrk_t(&c, &a, alpha, beta, uplo);
}

#define REF_TRI(name)                                                          \
  void ref_##name(mat_elem_t *x, const mat_elem_t *T, const mat_elem_t *b,    \
                  size_t n) {                                                  \
    Mat xv = wrap(n, 1, x), t = wrap(n, n, T), bv = wrap(n, 1, b);             \
    mat_##name(&xv, &t, &bv);                                                  \
  }
REF_TRI(solve_tril)
REF_TRI(solve_tril_unit)
REF_TRI(solve_triu)
REF_TRI(solve_trilt)

void ref_solve(mat_elem_t *x, const mat_elem_t *A, const mat_elem_t *b,
               size_t n) {
  Mat xv = wrap(n, 1, x), a = wrap(n, n, A), bv = wrap(n, 1, b);
  mat_solve(&xv, &a, &bv);
}

int ref_solve_spd(mat_elem_t *x, const mat_elem_t *A, const mat_elem_t *b,
                  size_t n) {
  Mat xv = wrap(n, 1, x), a = wrap(n, n, A), bv = wrap(n, 1, b);
  return mat_solve_spd(&xv, &a, &bv);
}

void ref_gemv(mat_elem_t *y, mat_elem_t alpha, const mat_elem_t *A,
              const mat_elem_t *x, mat_elem_t beta, size_t m, size_t n) {
  Mat yv = wrap(m, 1, y), a = wrap(m, n, A), xv = wrap(n, 1, x);
  mat_gemv(&yv, alpha, &a, &xv, beta);
}

void ref_gemv_t(mat_elem_t *y, mat_elem_t alpha, const mat_elem_t *A,
                const mat_elem_t *x, mat_elem_t beta, size_t m, size_t n) {
  Mat yv = wrap(n, 1, y), a = wrap(m, n, A), xv = wrap(m, 1, x);
  mat_gemv_t(&yv, alpha, &a, &xv, beta);
}

void ref_axpy(mat_elem_t *y, mat_elem_t alpha, const mat_elem_t *x, size_t n) {
  Mat yv = wrap(n, 1, y), xv = wrap(n, 1, x);
  mat_axpy(&yv, alpha, &xv);
}

void ref_qr(const mat_elem_t *A, size_t m, size_t n, mat_elem_t *Q,
            mat_elem_t *R) {
  Mat a = wrap(m, n, A), q = wrap(m, m, Q), r = wrap(m, n, R);
  mat_qr(&a, &q, &r);
}

/* glibc rand() stream, so the reference tests' srand(42) fixtures can be
 * regenerated bit-for-bit by the fixture script. */
void ref_srand(unsigned s) { srand(s); }
int ref_rand(void) { return rand(); }
