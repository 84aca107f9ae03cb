// The mat.h hot-path entry points (C ABI, host Mat in and out).
//
// Each call: asserts exactly as the reference does, copies the host operands
// into the library's device workspace, runs the device routines on the
// library stream, copies the results back and synchronises.  No CPU compute
// path exists for any of them.
#include <stdlib.h>
#include <string.h>

#include <utility>
#include <vector>

#include "internal.cuh"

using namespace mgb;

namespace {

constexpr size_t ES = sizeof(elem_t);

int h2d(void *d, const void *h, size_t bytes) {
  if (bytes) MGB_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx()->stream));
  return 0;
}
int d2h(void *h, const void *d, size_t bytes) {
  if (bytes) MGB_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx()->stream));
  return 0;
}
int sync() {
  MGB_CUDA(cudaStreamSynchronize(ctx()->stream));
  if (lu_wait_error(1))
    return set_error(MATGB_ERR_TIMEOUT, "LU panel exchange gave up waiting");
  MGB_TRY(trsv_status());
  MGB_TRY(trsm_flag_status());
  return 0;
}

#define WS(ptr, type, slot, count)                                             \
  type *ptr = (type *)ws(slot, (size_t)(count) * sizeof(type));                \
  if (!ptr) return MATGB_ERR_NOMEM;

// L = unit lower part of W, U = upper part (mat_plu's split, mat.h:4456-4470).
__global__ void split_lu_kernel(int64_t n, const elem_t *__restrict__ W,
                                elem_t *__restrict__ L, elem_t *__restrict__ U) {
  const int64_t tot = n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n, j = e / n;
    const elem_t w = W[e];
    L[e] = i > j ? w : (i == j ? elem_t(1) : elem_t(0));
    U[e] = i <= j ? w : elem_t(0);
  }
}

// Zero the strict upper triangle (mat_chol's output has zeros there).
__global__ void zero_upper_kernel(int64_t n, elem_t *__restrict__ W) {
  const int64_t tot = n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x)
    if (e % n < e / n) W[e] = elem_t(0);
}

__global__ void eye_kernel(int64_t n, elem_t *__restrict__ W) {
  const int64_t tot = n * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x)
    W[e] = (e % n == e / n) ? elem_t(1) : elem_t(0);
}

__global__ void diag_kernel(int64_t n, const elem_t *__restrict__ W,
                            elem_t *__restrict__ d) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = W[i * n + i];
}

unsigned grid_elems(int64_t tot) {
  int64_t b = (tot + 255) / 256;
  int64_t cap = (int64_t)ctx()->sms * 16;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

int do_gemm(Mat *C, elem_t alpha, const Mat *A, const Mat *B, elem_t beta) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t m = A->rows, k = A->cols, n = B->cols;
  WS(dA, elem_t, WS_A, m * k);
  WS(dB, elem_t, WS_B, k * n);
  WS(dC, elem_t, WS_C, m * n);
  MGB_TRY(h2d(dA, A->data, m * k * ES));
  MGB_TRY(h2d(dB, B->data, k * n * ES));
  if (beta != elem_t(0)) MGB_TRY(h2d(dC, C->data, m * n * ES));
  MGB_TRY(gemm(false, false, m, n, k, alpha, dA, m, dB, k, beta, dC, m, 0));
  MGB_TRY(d2h(C->data, dC, m * n * ES));
  return sync();
}

int do_qr(const Mat *A, Mat *Q, Mat *R) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t m = A->rows, n = A->cols;
  WS(dR, elem_t, WS_A, m * n);
  elem_t *dQ = nullptr;
  if (Q) {
    dQ = (elem_t *)ws(WS_B, (size_t)(m * m) * sizeof(elem_t));
    if (!dQ) return MATGB_ERR_NOMEM;
  }
  MGB_TRY(h2d(dR, A->data, m * n * ES));
  MGB_TRY(qr(m, n, dR, m, dQ, m));
  MGB_TRY(d2h(R->data, dR, m * n * ES));
  if (Q) MGB_TRY(d2h(Q->data, dQ, m * m * ES));
  return sync();
}

int do_syrk(Mat *C, const Mat *A, elem_t alpha, elem_t beta, char uplo,
            bool trans) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = C->rows;
  const int64_t k = trans ? A->rows : A->cols;
  const int tri = (uplo == 'L' || uplo == 'l') ? 1 : 2;  // else: upper
  WS(dA, elem_t, WS_A, A->rows * A->cols);
  WS(dC, elem_t, WS_C, n * n);
  MGB_TRY(h2d(dA, A->data, A->rows * A->cols * ES));
  MGB_TRY(h2d(dC, C->data, n * n * ES));
  MGB_TRY(gemm(trans, !trans, n, n, k, alpha, dA, A->rows, dA, A->rows, beta,
               dC, n, tri));
  MGB_TRY(d2h(C->data, dC, n * n * ES));
  return sync();
}

int do_gemv(Vec *y, elem_t alpha, const Mat *A, const Vec *x, elem_t beta) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t m = A->rows, n = A->cols;
  WS(dA, elem_t, WS_A, m * n);
  WS(dx, elem_t, WS_B, n);
  WS(dy, elem_t, WS_C, m);
  MGB_TRY(h2d(dA, A->data, m * n * ES));
  MGB_TRY(h2d(dx, x->data, n * ES));
  if (beta != elem_t(0)) MGB_TRY(h2d(dy, y->data, m * ES));
  MGB_TRY(gemv(m, n, alpha, dA, m, dx, beta, dy));
  MGB_TRY(d2h(y->data, dy, m * ES));
  return sync();
}

int do_gemv_t(Vec *y, elem_t alpha, const Mat *A, const Vec *x, elem_t beta) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t m = A->rows, n = A->cols;
  WS(dA, elem_t, WS_A, m * n);
  WS(dx, elem_t, WS_B, m);
  WS(dy, elem_t, WS_C, n);
  MGB_TRY(h2d(dA, A->data, m * n * ES));
  MGB_TRY(h2d(dx, x->data, m * ES));
  MGB_TRY(h2d(dy, y->data, n * ES));  // read even for beta = 0, as mat.h:2235
  MGB_TRY(gemv_t_t<elem_t>(m, n, alpha, dA, m, dx, beta, dy));
  MGB_TRY(d2h(y->data, dy, n * ES));
  return sync();
}

int do_axpy(Vec *y, elem_t alpha, const Vec *x) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = x->rows;
  WS(dx, elem_t, WS_B, n);
  WS(dy, elem_t, WS_C, n);
  MGB_TRY(h2d(dx, x->data, n * ES));
  MGB_TRY(h2d(dy, y->data, n * ES));
  MGB_TRY(axpy_t<elem_t>(n, alpha, dx, dy));
  MGB_TRY(d2h(y->data, dy, n * ES));
  return sync();
}

// Factor a host matrix on the device; leaves the packed LU in WS_A and
// ipiv|perm in WS_PIV.  Returns the device pointers.
int factor_lu(const Mat *A, elem_t **W_out, int32_t **piv_out) {
  const int64_t n = A->rows;
  WS(W, elem_t, WS_A, n * n);
  WS(piv, int32_t, WS_PIV, 2 * n);
  MGB_TRY(h2d(W, A->data, n * n * ES));
  MGB_TRY(getrf(n, W, n, piv, piv + n));
  *W_out = W;
  *piv_out = piv;
  return 0;
}

int count_swaps(const std::vector<int32_t> &ipiv, int64_t n) {
  int s = 0;
  for (int64_t k = 0; k + 1 < n; k++) s += (ipiv[k] != k);
  return s;
}

int do_plu(const Mat *A, Mat *L, Mat *U, Perm *p, int *swaps) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows;
  elem_t *W;
  int32_t *piv;
  MGB_TRY(factor_lu(A, &W, &piv));
  WS(dL, elem_t, WS_L, n * n);
  WS(dU, elem_t, WS_U, n * n);
  split_lu_kernel<<<grid_elems(n * n), 256, 0, ctx()->stream>>>(n, W, dL, dU);
  MGB_LAUNCHED("split_lu");
  std::vector<int32_t> hp(2 * n);
  MGB_TRY(d2h(L->data, dL, n * n * ES));
  MGB_TRY(d2h(U->data, dU, n * n * ES));
  MGB_TRY(d2h(hp.data(), piv, 2 * n * sizeof(int32_t)));
  MGB_TRY(sync());
  for (int64_t i = 0; i < n; i++) p->data[i] = (size_t)hp[n + i];
  *swaps = count_swaps(hp, n);
  return 0;
}

// Full pivoting (mat_lu): eliminate on the device, split L and U there, and
// replay the recorded swaps on the host into p, q and the swap count, in the
// reference's order (rows, then columns; mat.h:4476-4574).
int do_lu(const Mat *A, Mat *L, Mat *U, Perm *p, Perm *q, int *swaps) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows;
  for (int64_t i = 0; i < n; i++) p->data[i] = q->data[i] = (size_t)i;
  *swaps = 0;
  if (n == 0) return 0;
  WS(W, elem_t, WS_A, n * n);
  WS(piv, int32_t, WS_PIV, 2 * n);
  WS(dL, elem_t, WS_L, n * n);
  WS(dU, elem_t, WS_U, n * n);
  MGB_TRY(h2d(W, A->data, n * n * ES));
  MGB_TRY(getrf_full_t<elem_t>(n, W, n, piv, piv + n, kPivotEps));
  split_lu_kernel<<<grid_elems(n * n), 256, 0, ctx()->stream>>>(n, W, dL, dU);
  MGB_LAUNCHED("split_lu");
  std::vector<int32_t> hp(2 * n);
  MGB_TRY(d2h(L->data, dL, n * n * ES));
  MGB_TRY(d2h(U->data, dU, n * n * ES));
  MGB_TRY(d2h(hp.data(), piv, 2 * n * sizeof(int32_t)));
  MGB_TRY(sync());
  for (int64_t k = 0; k + 1 < n; k++) {
    const int64_t pr = hp[k], pc = hp[n + k];
    if (pr != k) {
      std::swap(p->data[k], p->data[pr]);
      ++*swaps;
    }
    if (pc != k) {
      std::swap(q->data[k], q->data[pc]);
      ++*swaps;
    }
  }
  return 0;
}

int do_det(const Mat *A, elem_t *det) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows;
  elem_t *W;
  int32_t *piv;
  MGB_TRY(factor_lu(A, &W, &piv));
  WS(dd, elem_t, WS_X, n);
  diag_kernel<<<grid_elems(n), 256, 0, ctx()->stream>>>(n, W, dd);
  MGB_LAUNCHED("diag");
  std::vector<elem_t> hd(n);
  std::vector<int32_t> hp(n);
  MGB_TRY(d2h(hd.data(), dd, n * ES));
  MGB_TRY(d2h(hp.data(), piv, n * sizeof(int32_t)));
  MGB_TRY(sync());
  // det = (-1)^swaps * prod(diag U), in the reference's order (mat.h:6236-6242)
  elem_t d = (count_swaps(hp, n) % 2 == 0) ? 1 : -1;
  for (int64_t i = 0; i < n; i++) d *= hd[i];
  *det = d;
  return 0;
}

int do_inv(Mat *out, const Mat *A) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows;
  elem_t *W;
  int32_t *piv;
  MGB_TRY(factor_lu(A, &W, &piv));
  WS(I, elem_t, WS_B, n * n);
  WS(X, elem_t, WS_X, n * n);
  eye_kernel<<<grid_elems(n * n), 256, 0, ctx()->stream>>>(n, I);
  MGB_LAUNCHED("eye");
  MGB_TRY(getrs(n, n, W, n, piv + n, I, n, X, n));
  MGB_TRY(d2h(out->data, X, n * n * ES));
  return sync();
}

int do_solve(Mat *X, const Mat *A, const Mat *B, int64_t nrhs) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows;
  elem_t *W;
  int32_t *piv;
  MGB_TRY(factor_lu(A, &W, &piv));
  WS(dB, elem_t, WS_B, n * nrhs);
  WS(dX, elem_t, WS_X, n * nrhs);
  // Column c of B starts at c*B->rows (only the first n rows are read).
  for (int64_t c = 0; c < nrhs; c++)
    MGB_TRY(h2d(dB + c * n, B->data + c * B->rows, n * ES));
  MGB_TRY(getrs(n, nrhs, W, n, piv + n, dB, n, dX, n));
  for (int64_t c = 0; c < nrhs; c++)
    MGB_TRY(d2h(X->data + c * X->rows, dX + c * n, n * ES));
  return sync();
}

// Returns 0, or -1 when A is not positive definite (X untouched then).
int do_solve_spd(Mat *X, const Mat *A, const Mat *B, int64_t nrhs, int *ret) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows;
  WS(W, elem_t, WS_A, n * n);
  WS(info, int32_t, WS_INFO, 1);
  WS(dX, elem_t, WS_X, n * nrhs);
  MGB_TRY(h2d(W, A->data, n * n * ES));
  for (int64_t c = 0; c < nrhs; c++)
    MGB_TRY(h2d(dX + c * n, B->data + c * B->rows, n * ES));
  MGB_TRY(potrf(n, W, n, info));
  MGB_TRY(potrs(n, nrhs, W, n, dX, n, info));
  int32_t hinfo = 0;
  MGB_TRY(d2h(&hinfo, info, sizeof hinfo));
  MGB_TRY(sync());
  if (hinfo != 0) {
    *ret = -1;
    return 0;
  }
  for (int64_t c = 0; c < nrhs; c++)
    MGB_TRY(d2h(X->data + c * X->rows, dX + c * n, n * ES));
  MGB_TRY(sync());
  *ret = 0;
  return 0;
}

int do_chol(const Mat *A, Mat *L, int *ret) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows;
  WS(W, elem_t, WS_A, n * n);
  WS(info, int32_t, WS_INFO, 1);
  MGB_TRY(h2d(W, A->data, n * n * ES));
  MGB_TRY(potrf(n, W, n, info));
  zero_upper_kernel<<<grid_elems(n * n), 256, 0, ctx()->stream>>>(n, W);
  MGB_LAUNCHED("zero_upper");
  int32_t hinfo = 0;
  MGB_TRY(d2h(L->data, W, n * n * ES));
  MGB_TRY(d2h(&hinfo, info, sizeof hinfo));
  MGB_TRY(sync());
  *ret = hinfo == 0 ? 0 : -1;
  return 0;
}

int do_tri(Vec *x, const Mat *T, const Vec *b, bool lower, bool trans,
           bool unit) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = T->rows;
  WS(dT, elem_t, WS_A, n * n);
  WS(dx, elem_t, WS_X, n);
  MGB_TRY(h2d(dT, T->data, n * n * ES));
  MGB_TRY(h2d(dx, b->data, n * ES));
  MGB_TRY(trsm_left(lower, trans, unit, n, 1, dT, n, dx, n, nullptr));
  MGB_TRY(d2h(x->data, dx, n * ES));
  return sync();
}

}  // namespace

extern "C" {

void mat_gemm(Mat *C, mat_elem_t alpha, const Mat *A, const Mat *B,
              mat_elem_t beta) {  // mat.h:2787-2796
  MAT_ASSERT_MAT(C);
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(B);
  MAT_ASSERT(A->cols == B->rows);
  MAT_ASSERT(C->rows == A->rows && C->cols == B->cols);
  if (do_gemm(C, alpha, A, B, beta)) fail_void("mat_gemm");
}

void mat_mul(Mat *out, const Mat *a, const Mat *b) {  // mat.h:1842-1850
  MAT_ASSERT_MAT(out);
  MAT_ASSERT_MAT(a);
  MAT_ASSERT_MAT(b);
  MAT_ASSERT(a->cols == b->rows);
  mat_gemm(out, 1, a, b, 0);
}

Mat *mat_rmul(const Mat *a, const Mat *b) {  // mat.h:1852-1862
  MAT_ASSERT_MAT(a);
  MAT_ASSERT_MAT(b);
  MAT_ASSERT(a->cols == b->rows);
  Mat *r = mat_mat(a->rows, b->cols);
  mat_mul(r, a, b);
  return r;
}

void mat_gemv(Vec *y, mat_elem_t alpha, const Mat *A, const Vec *x,
              mat_elem_t beta) {  // mat.h:2137-2146
  MAT_ASSERT_MAT(y);
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(x);
  MAT_ASSERT(A->rows == y->rows);
  MAT_ASSERT(A->cols == x->rows);
  if (do_gemv(y, alpha, A, x, beta)) fail_void("mat_gemv");
}

void mat_gemv_t(Vec *y, mat_elem_t alpha, const Mat *A, const Vec *x,
                mat_elem_t beta) {  // mat.h:2239-2248
  MAT_ASSERT_MAT(y);
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(x);
  MAT_ASSERT(A->cols == y->rows);
  MAT_ASSERT(A->rows == x->rows);
  if (do_gemv_t(y, alpha, A, x, beta)) fail_void("mat_gemv_t");
}

void mat_axpy(Vec *y, mat_elem_t alpha, const Vec *x) {  // mat.h:2009-2015
  MAT_ASSERT_MAT(y);
  MAT_ASSERT_MAT(x);
  MAT_ASSERT(y->rows == x->rows);
  if (do_axpy(y, alpha, x)) fail_void("mat_axpy");
}

void mat_syrk(Mat *C, const Mat *A, mat_elem_t alpha, mat_elem_t beta,
              char uplo) {  // mat.h:5670-5679
  MAT_ASSERT_MAT(C);
  MAT_ASSERT_MAT(A);
  MAT_ASSERT(C->rows == C->cols);
  MAT_ASSERT(C->rows == A->rows);
  if (do_syrk(C, A, alpha, beta, uplo, false)) fail_void("mat_syrk");
}

void mat_syrk_t(Mat *C, const Mat *A, mat_elem_t alpha, mat_elem_t beta,
                char uplo) {  // mat.h:5727-5735
  MAT_ASSERT_MAT(C);
  MAT_ASSERT_MAT(A);
  MAT_ASSERT(C->rows == C->cols);
  MAT_ASSERT(C->rows == A->cols);
  if (do_syrk(C, A, alpha, beta, uplo, true)) fail_void("mat_syrk_t");
}

int mat_plu(const Mat *A, Mat *L, Mat *U, Perm *p) {  // mat.h:4436-4474
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(L);
  MAT_ASSERT_MAT(U);
  MAT_ASSERT(p != NULL);
  MAT_ASSERT_SQUARE(A);
  size_t n = A->rows;
  MAT_ASSERT(L->rows == n && L->cols == n);
  MAT_ASSERT(U->rows == n && U->cols == n);
  MAT_ASSERT(p->size == n);
  int swaps = 0;
  if (do_plu(A, L, U, p, &swaps)) {
    fail_void("mat_plu");
    return -1;
  }
  return swaps;
}

int mat_chol(const Mat *A, Mat *L) {  // mat.h:6062-6092
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(L);
  MAT_ASSERT_SQUARE(A);
  size_t n = A->rows;
  MAT_ASSERT(L->rows == n && L->cols == n);
  int ret = -1;
  if (do_chol(A, L, &ret)) {
    fail_void("mat_chol");
    return -1;
  }
  return ret;
}

int mat_lu(const Mat *A, Mat *L, Mat *U, Perm *p, Perm *q) {  // mat.h:4476
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(L);
  MAT_ASSERT_MAT(U);
  MAT_ASSERT(p != NULL && q != NULL);
  MAT_ASSERT_SQUARE(A);
  size_t n = A->rows;
  MAT_ASSERT(L->rows == n && L->cols == n);
  MAT_ASSERT(U->rows == n && U->cols == n);
  MAT_ASSERT(p->size == n && q->size == n);
  int swaps = 0;
  if (do_lu(A, L, U, p, q, &swaps)) {
    fail_void("mat_lu");
    return -1;
  }
  return swaps;
}

mat_elem_t mat_det(const Mat *A) {  // mat.h:6227-6249
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_SQUARE(A);
  elem_t d = 0;
  if (do_det(A, &d)) fail_void("mat_det");
  return d;
}

void mat_inv(Mat *out, const Mat *A) {  // mat.h:6166-6225
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(out);
  MAT_ASSERT_SQUARE(A);
  size_t n = A->rows;
  MAT_ASSERT(out->rows == n && out->cols == n);
  if (do_inv(out, A)) fail_void("mat_inv");
}

void mat_qr(const Mat *A, Mat *Q, Mat *R) {  // mat.h:3907-4064
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(Q);
  MAT_ASSERT_MAT(R);
  const size_t m = A->rows, n = A->cols;
  MAT_ASSERT(m >= n && "mat_qr requires m >= n");
  MAT_ASSERT(Q->rows == m && Q->cols == m);
  MAT_ASSERT(R->rows == m && R->cols == n);
  if (do_qr(A, Q, R)) fail_void("mat_qr");
}

void mat_qr_r(const Mat *A, Mat *R) {  // mat.h:4066-4192
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(R);
  const size_t m = A->rows, n = A->cols;
  MAT_ASSERT(m >= n && "mat_qr_r requires m >= n");
  MAT_ASSERT(R->rows == m && R->cols == n);
  if (do_qr(A, nullptr, R)) fail_void("mat_qr_r");
}

void mat_solve(Vec *x, const Mat *A, const Vec *b) {  // mat.h:4807-4837
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(x);
  MAT_ASSERT_MAT(b);
  MAT_ASSERT_SQUARE(A);
  MAT_ASSERT(b->rows == A->rows && "b must have same rows as A");
  MAT_ASSERT(x->rows == A->cols && "x must have same rows as A cols");
  if (do_solve(x, A, b, 1)) fail_void("mat_solve");
}

int mat_solve_spd(Vec *x, const Mat *A, const Vec *b) {  // mat.h:4839-4871
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(x);
  MAT_ASSERT_MAT(b);
  MAT_ASSERT_SQUARE(A);
  MAT_ASSERT(b->rows == A->rows && "b must have same rows as A");
  MAT_ASSERT(x->rows == A->cols && "x must have same rows as A cols");
  int ret = -1;
  if (do_solve_spd(x, A, b, 1, &ret)) {
    fail_void("mat_solve_spd");
    return -1;
  }
  return ret;
}

#define MGB_TRI_ASSERTS(T)                                                     \
  MAT_ASSERT_MAT(T);                                                           \
  MAT_ASSERT_MAT(x);                                                           \
  MAT_ASSERT_MAT(b);                                                           \
  MAT_ASSERT_SQUARE(T);                                                        \
  MAT_ASSERT(b->rows == T->rows);                                              \
  MAT_ASSERT(x->rows == T->rows)

void mat_solve_tril(Vec *x, const Mat *L, const Vec *b) {  // mat.h:4626-4634
  MGB_TRI_ASSERTS(L);
  if (do_tri(x, L, b, true, false, false)) fail_void("mat_solve_tril");
}

void mat_solve_tril_unit(Vec *x, const Mat *L, const Vec *b) {  // :4679-4687
  MGB_TRI_ASSERTS(L);
  if (do_tri(x, L, b, true, false, true)) fail_void("mat_solve_tril_unit");
}

void mat_solve_triu(Vec *x, const Mat *U, const Vec *b) {  // mat.h:4738-4746
  MGB_TRI_ASSERTS(U);
  if (do_tri(x, U, b, false, false, false)) fail_void("mat_solve_triu");
}

void mat_solve_trilt(Vec *x, const Mat *L, const Vec *b) {  // mat.h:4792-4803
  MGB_TRI_ASSERTS(L);
  if (do_tri(x, L, b, true, true, false)) fail_void("mat_solve_trilt");
}

void matgb_solve_multi(Mat *X, const Mat *A, const Mat *B) {
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(X);
  MAT_ASSERT_MAT(B);
  MAT_ASSERT_SQUARE(A);
  MAT_ASSERT(B->rows == A->rows && X->rows == A->cols);
  MAT_ASSERT(X->cols == B->cols);
  if (do_solve(X, A, B, (int64_t)B->cols)) fail_void("matgb_solve_multi");
}

int matgb_solve_spd_multi(Mat *X, const Mat *A, const Mat *B) {
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(X);
  MAT_ASSERT_MAT(B);
  MAT_ASSERT_SQUARE(A);
  MAT_ASSERT(B->rows == A->rows && X->rows == A->cols);
  MAT_ASSERT(X->cols == B->cols);
  int ret = -1;
  if (do_solve_spd(X, A, B, (int64_t)B->cols, &ret)) {
    fail_void("matgb_solve_spd_multi");
    return -1;
  }
  return ret;
}

}  // extern "C"
