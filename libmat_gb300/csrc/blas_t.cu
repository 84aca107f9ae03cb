// Transposed matrix-vector product and AXPY:
//   y[j] = beta * y[j] + alpha * dot(A[:, j], x)   (mat_gemv_t, mat.h:2224-2248)
//   y[i] += alpha * x[i]                           (mat_axpy, mat.h:2009-2015)
//
// Both stream their operands once and are bound by HBM.  The transposed
// product reads A (m x n, column-major) one column per warp: each column is
// contiguous, x stays in L2.  With too few columns to fill the GPU the rows
// are split into chunks, each (chunk, column) pair a warp, and a second
// launch adds the chunks' partial dots in chunk order, so the result does
// not depend on scheduling.  The final combination rounds as the reference
// does: beta * y and alpha * dot rounded separately, then their sum.  AXPY
// rounds alpha * x[i] before the addition, as the reference's scalar loop
// compiled without contraction; its results are bit-identical.
#include <algorithm>

#include "internal.cuh"

namespace mgb {
namespace {

constexpr int kTvWarps = 8;      // warps (columns) per CTA
constexpr int kTvUnroll = 8;     // loads in flight per thread
constexpr int64_t kTvChunk = 8192;  // fewest rows per chunk when the rows are split

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// Partial dot of rows [i0, i1) of column j with x.
template <typename T>
__device__ T column_dot(const T *__restrict__ col, const T *__restrict__ x,
                        int64_t i0, int64_t i1, int lane) {
  T acc[kTvUnroll];
#pragma unroll
  for (int u = 0; u < kTvUnroll; u++) acc[u] = T(0);
  int64_t i = i0 + lane;
  for (; i + (kTvUnroll - 1) * 32 < i1; i += kTvUnroll * 32) {
    T a[kTvUnroll], b[kTvUnroll];
#pragma unroll
    for (int u = 0; u < kTvUnroll; u++) {
      a[u] = __ldcs(col + i + u * 32);  // streamed once
      b[u] = x[i + u * 32];
    }
#pragma unroll
    for (int u = 0; u < kTvUnroll; u++) acc[u] += a[u] * b[u];
  }
  for (; i < i1; i += 32) acc[0] += col[i] * x[i];
  T s = T(0);
#pragma unroll
  for (int u = 0; u < kTvUnroll; u++) s += acc[u];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// chunks == 1: y[j] = beta*y[j] + alpha*dot.  chunks > 1: part[c*n + j] =
// the dot over rows [c*rpc, (c+1)*rpc) (chunk c = blockIdx.y), where
// chunks * rpc >= m.
template <typename T>
__global__ void __launch_bounds__(kTvWarps * 32)
    gemv_t_kernel(int64_t m, int64_t n, T alpha, const T *__restrict__ A,
                  int64_t lda, const T *__restrict__ x, T beta,
                  T *__restrict__ y, T *__restrict__ part, int chunks,
                  int64_t rpc) {
  const int lane = threadIdx.x & 31;
  const int64_t j = (int64_t)blockIdx.x * kTvWarps + (threadIdx.x >> 5);
  if (j >= n) return;
  const int64_t c = blockIdx.y;
  const int64_t i0 = chunks == 1 ? 0 : c * rpc;
  const int64_t i1 = chunks == 1 ? m : (i0 + rpc < m ? i0 + rpc : m);
  const T d = column_dot(A + j * lda, x, i0, i1, lane);
  if (lane != 0) return;
  if (chunks == 1)
    y[j] = add_rn(mul_rn(beta, y[j]), mul_rn(alpha, d));
  else
    part[c * n + j] = d;
}

template <typename T>
__global__ void gemv_t_reduce_kernel(int64_t n, int chunks, T alpha,
                                     const T *__restrict__ part, T beta,
                                     T *__restrict__ y) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    T d = T(0);
    for (int c = 0; c < chunks; c++) d += part[(int64_t)c * n + j];
    y[j] = add_rn(mul_rn(beta, y[j]), mul_rn(alpha, d));
  }
}

template <typename T>
__global__ void axpy_kernel(int64_t n, T alpha, const T *__restrict__ x,
                            T *__restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = add_rn(y[i], mul_rn(alpha, __ldcs(x + i)));
}

}  // namespace

template <typename T>
int gemv_t_t(int64_t m, int64_t n, T alpha, const T *A, int64_t lda,
             const T *x, T beta, T *y) {
  if (n <= 0) return 0;
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  cudaStream_t s = cx->stream;
  const int64_t cols = (n + kTvWarps - 1) / kTvWarps;
  // split the rows when the columns alone give under ~4 CTAs per SM
  int chunks = 1;
  int64_t rpc = m;  // rows per chunk
  const int64_t want = (int64_t)cx->sms * 4;
  if (cols < want && m > 2 * kTvChunk) {
    const int64_t c0 = std::min<int64_t>((m + kTvChunk - 1) / kTvChunk,
                                         (want + cols - 1) / cols);
    rpc = ((m + c0 - 1) / c0 + 255) / 256 * 256;
    chunks = (int)((m + rpc - 1) / rpc);  // every row in exactly one chunk
  }
  T *part = nullptr;
  if (chunks > 1) {
    part = (T *)ws(WS_K, (size_t)chunks * n * sizeof(T));
    if (!part) return MATGB_ERR_NOMEM;
  }
  KtScope kt("gemv_t", 2.0 * m * n, (double)sizeof(T) * (m * n + m + 2 * n));
  gemv_t_kernel<T><<<dim3((unsigned)cols, (unsigned)chunks), kTvWarps * 32, 0,
                     s>>>(m, n, alpha, A, lda, x, beta, y, part, chunks, rpc);
  MGB_LAUNCHED("gemv_t");
  if (chunks > 1) {
    gemv_t_reduce_kernel<T><<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024),
                              256, 0, s>>>(n, chunks, alpha, part, beta, y);
    MGB_LAUNCHED("gemv_t_reduce");
  }
  return 0;
}

template <typename T>
int axpy_t(int64_t n, T alpha, const T *x, T *y) {
  if (n <= 0) return 0;
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  const unsigned grid =
      (unsigned)std::min<int64_t>((n + 255) / 256, (int64_t)cx->sms * 16);
  KtScope kt("axpy", 2.0 * n, 3.0 * sizeof(T) * n);
  axpy_kernel<T><<<grid, 256, 0, cx->stream>>>(n, alpha, x, y);
  MGB_LAUNCHED("axpy");
  return 0;
}

template int gemv_t_t<elem_t>(int64_t, int64_t, elem_t, const elem_t *,
                              int64_t, const elem_t *, elem_t, elem_t *);
template int axpy_t<elem_t>(int64_t, elem_t, const elem_t *, elem_t *);

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_gemv_t_dev(size_t m, size_t n, mat_elem_t alpha, const mat_elem_t *A,
                     size_t lda, const mat_elem_t *x, mat_elem_t beta,
                     mat_elem_t *y) {
  if (lda < m) return set_error(MATGB_ERR_ARG, "gemv_t: lda < m");
  return gemv_t_t<elem_t>((int64_t)m, (int64_t)n, alpha, A, (int64_t)lda, x,
                          beta, y);
}

int matgb_axpy_dev(size_t n, mat_elem_t alpha, const mat_elem_t *x,
                   mat_elem_t *y) {
  return axpy_t<elem_t>((int64_t)n, alpha, x, y);
}

}  // extern "C"
