// SIMT GEMM / SYRK / GEMV in the library's element type (float or double).
// (Large float products go to the tensor cores instead: tc_sgemm.cu.)
//
// This is the plain-precision path: mat_gemm / mat_mul, the LU trailing
// update A22 -= L21*U12 (mat__gemm_strided_, mat.h:2719-2741, called from
// mat.h:4277-4283), the Cholesky SYRK update (mat__syrk_lower_,
// mat.h:5474-5486) and the triangular-solve block updates.  FP32/FP64 are not
// tensor-core types on sm_103a (tcgen05 has no f32/f64 kind), so the plain path
// is an FFMA/DFMA register-tiled kernel: CTA tile BM x BN, K step BK staged in
// shared memory (double buffered through registers), TM x TN accumulators per
// thread, column-major operands with optional transposes, optional
// lower/upper-triangle masking for SYRK.
#include "internal.cuh"

namespace mgb {

template <typename T>
struct GemmCfg;
template <>
struct GemmCfg<float> {
  static constexpr int BM = 128, BN = 128, BK = 16, TM = 8, TN = 8;
};
template <>
struct GemmCfg<double> {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
};

template <typename T, int BM, int BN, int BK, int TM, int TN, bool TA, bool TB,
          int TRI>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    gemm_kernel(int64_t M, int64_t N, int64_t K, T alpha,
                const T *__restrict__ A, int64_t lda, const T *__restrict__ B,
                int64_t ldb, T beta, T *__restrict__ C, int64_t ldc,
                const int32_t *__restrict__ skip) {
  constexpr int RT = BM / TM;  // threads along M
  constexpr int NT = RT * (BN / TN);
  constexpr int LA = BM * BK / NT;
  constexpr int LB = BK * BN / NT;
  static_assert(LA * NT == BM * BK && LB * NT == BK * BN, "tile split");
  __shared__ __align__(16) T As[2][BK][BM + 4];
  __shared__ __align__(16) T Bs[2][BK][BN + 4];

  if (skip && *skip != 0) return;
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  if (TRI == 1 && n0 >= m0 + BM) return;  // tile strictly above diagonal
  if (TRI == 2 && m0 >= n0 + BN) return;  // tile strictly below diagonal

  const int tid = threadIdx.x;
  const int tr = tid % RT;  // consecutive threads walk down a column of C
  const int tc = tid / RT;

  T ra[LA], rb[LB];
  auto load_regs = [&](int64_t k0) {
#pragma unroll
    for (int r = 0; r < LA; r++) {
      int e = tid + r * NT;
      int i, kk;
      if (!TA) { i = e % BM; kk = e / BM; } else { kk = e % BK; i = e / BK; }
      int64_t gi = m0 + i, gk = k0 + kk;
      T v = T(0);
      if (gi < M && gk < K) v = TA ? A[gi * lda + gk] : A[gk * lda + gi];
      ra[r] = v;
    }
#pragma unroll
    for (int r = 0; r < LB; r++) {
      int e = tid + r * NT;
      int j, kk;
      if (!TB) { kk = e % BK; j = e / BK; } else { j = e % BN; kk = e / BN; }
      int64_t gj = n0 + j, gk = k0 + kk;
      T v = T(0);
      if (gj < N && gk < K) v = TB ? B[gk * ldb + gj] : B[gj * ldb + gk];
      rb[r] = v;
    }
  };
  auto store_smem = [&](int buf) {
#pragma unroll
    for (int r = 0; r < LA; r++) {
      int e = tid + r * NT;
      int i, kk;
      if (!TA) { i = e % BM; kk = e / BM; } else { kk = e % BK; i = e / BK; }
      As[buf][kk][i] = ra[r];
    }
#pragma unroll
    for (int r = 0; r < LB; r++) {
      int e = tid + r * NT;
      int j, kk;
      if (!TB) { kk = e % BK; j = e / BK; } else { j = e % BN; kk = e / BN; }
      Bs[buf][kk][j] = rb[r];
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) acc[i][j] = T(0);

  if (K > 0) {
    load_regs(0);
    store_smem(0);
  }
  __syncthreads();
  for (int64_t k0 = 0; k0 < K; k0 += BK) {
    const int cur = (int)((k0 / BK) & 1);
    const bool more = k0 + BK < K;
    if (more) load_regs(k0 + BK);
#pragma unroll
    for (int kk = 0; kk < BK; kk++) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; i++) a[i] = As[cur][kk][tr * TM + i];
#pragma unroll
      for (int j = 0; j < TN; j++) b[j] = Bs[cur][kk][tc * TN + j];
#pragma unroll
      for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    if (more) store_smem(cur ^ 1);
    __syncthreads();
  }

#pragma unroll
  for (int j = 0; j < TN; j++) {
    const int64_t gj = n0 + tc * TN + j;
    if (gj >= N) continue;
#pragma unroll
    for (int i = 0; i < TM; i++) {
      const int64_t gi = m0 + tr * TM + i;
      if (gi >= M) continue;
      if (TRI == 1 && gi < gj) continue;
      if (TRI == 2 && gi > gj) continue;
      T *c = &C[gj * ldc + gi];
      T v = alpha * acc[i][j];
      if (beta != T(0)) v = beta * (*c) + v;
      *c = v;
    }
  }
}

template <typename T, bool TA, bool TB, int TRI>
static int launch_gemm(int64_t m, int64_t n, int64_t k, T alpha, const T *A,
                       int64_t lda, const T *B, int64_t ldb, T beta, T *C,
                       int64_t ldc, const int32_t *skip) {
  using G = GemmCfg<T>;
  Ctx *c = ctx();
  dim3 grid((unsigned)((m + G::BM - 1) / G::BM),
            (unsigned)((n + G::BN - 1) / G::BN));
  constexpr int threads = (G::BM / G::TM) * (G::BN / G::TN);
  const double fl = 2.0 * m * n * k * (TRI ? 0.5 : 1.0);
  const double by = (double)sizeof(T) *
                    (m * k + k * n + (beta != T(0) ? 2.0 : 1.0) * m * n *
                                         (TRI ? 0.5 : 1.0));
  KtScope kt(sizeof(T) == 4 ? "gemm_simt_f32" : "gemm_simt_f64", fl, by);
  gemm_kernel<T, G::BM, G::BN, G::BK, G::TM, G::TN, TA, TB, TRI>
      <<<grid, threads, 0, c->stream>>>(m, n, k, alpha, A, lda, B, ldb, beta,
                                        C, ldc, skip);
  MGB_LAUNCHED("gemm_simt");
  return 0;
}

template <typename T>
int gemm_skip_t(bool ta, bool tb, int64_t m, int64_t n, int64_t k, T alpha,
                const T *A, int64_t lda, const T *B, int64_t ldb, T beta, T *C,
                int64_t ldc, int tri, const int32_t *skip) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  if (m <= 0 || n <= 0) return 0;
#define MGB_G(TA_, TB_, TRI_)                                                  \
  if (ta == TA_ && tb == TB_ && tri == TRI_)                                   \
    return launch_gemm<T, TA_, TB_, TRI_>(m, n, k, alpha, A, lda, B, ldb,      \
                                          beta, C, ldc, skip);
  MGB_G(false, false, 0)
  MGB_G(true, false, 0)
  MGB_G(false, true, 0)
  MGB_G(true, true, 0)
  MGB_G(false, true, 1)
  MGB_G(false, true, 2)
  MGB_G(true, false, 1)
  MGB_G(true, false, 2)
#undef MGB_G
  return set_error(MATGB_ERR_ARG, "gemm: unsupported variant");
}

template int gemm_skip_t<float>(bool, bool, int64_t, int64_t, int64_t, float,
                                const float *, int64_t, const float *, int64_t,
                                float, float *, int64_t, int, const int32_t *);
template int gemm_skip_t<double>(bool, bool, int64_t, int64_t, int64_t, double,
                                 const double *, int64_t, const double *,
                                 int64_t, double, double *, int64_t, int,
                                 const int32_t *);

int gemm_skip(bool ta, bool tb, int64_t m, int64_t n, int64_t k, elem_t alpha,
              const elem_t *A, int64_t lda, const elem_t *B, int64_t ldb,
              elem_t beta, elem_t *C, int64_t ldc, int tri,
              const int32_t *skip) {
  return gemm_skip_t<elem_t>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C,
                             ldc, tri, skip);
}

// The public products (mat_mul, mat_gemm, mat_syrk, matgb_gemm_dev,
// matgb_syrk_dev): in the float build, products of at least 256 x 256 run on
// the tensor cores in the FP32-accurate split form (tc_sgemm.cu) unless
// matgb_plain_tensor_core(0) chose the SIMT kernel.
int gemm(bool ta, bool tb, int64_t m, int64_t n, int64_t k, elem_t alpha,
         const elem_t *A, int64_t lda, const elem_t *B, int64_t ldb,
         elem_t beta, elem_t *C, int64_t ldc, int tri) {
#ifndef MAT_DOUBLE_PRECISION
  if (plain_tc_on() && m >= kPlainTcMinMN && n >= kPlainTcMinMN && k >= 16) {
    // SYRK (op(B) = op(A)^T): one packed operand serves both sides
    const bool same_ab = A == B && lda == ldb && ta != tb && m == n;
    return tc_sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri,
                    same_ab);
  }
#endif
  return gemm_skip(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri,
                   nullptr);
}

// ---- GEMV: y = alpha*A*x + beta*y, column-major A (m x n) -----------------
// Column-split partial sums into a workspace, then a fixed-order reduction,
// so the result does not depend on scheduling.
constexpr int kGemvRows = 256;

template <typename T>
__global__ void __launch_bounds__(kGemvRows)
    gemv_partial_kernel(int64_t m, int64_t n, int64_t cols_per,
                        const T *__restrict__ A, int64_t lda,
                        const T *__restrict__ x, T *__restrict__ P) {
  const int64_t i = (int64_t)blockIdx.x * kGemvRows + threadIdx.x;
  const int64_t j0 = (int64_t)blockIdx.y * cols_per;
  int64_t j1 = j0 + cols_per;
  if (j1 > n) j1 = n;
  if (i >= m) return;
  T s = 0;
  for (int64_t j = j0; j < j1; j++) s = fma(A[j * lda + i], x[j], s);
  P[(int64_t)blockIdx.y * m + i] = s;
}

template <typename T>
__global__ void gemv_reduce_kernel(int64_t m, int chunks, T alpha,
                                   const T *__restrict__ P, T beta,
                                   T *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  T s = 0;
  for (int c = 0; c < chunks; c++) s += P[(int64_t)c * m + i];
  T v = alpha * s;
  if (beta != T(0)) v = beta * y[i] + v;
  y[i] = v;
}

template <typename T>
int gemv_t(int64_t m, int64_t n, T alpha, const T *A, int64_t lda, const T *x,
           T beta, T *y) {
  Ctx *c = ctx();
  if (!c) return MATGB_ERR_NO_DEVICE;
  if (m <= 0) return 0;
  int64_t rb = (m + kGemvRows - 1) / kGemvRows;
  int64_t target = (int64_t)c->sms * 8;
  int64_t chunks = (target + rb - 1) / rb;
  if (chunks > n) chunks = n > 0 ? n : 1;
  if (chunks > 1024) chunks = 1024;
  int64_t cols_per = n > 0 ? (n + chunks - 1) / chunks : 0;
  chunks = cols_per > 0 ? (n + cols_per - 1) / cols_per : 1;
  T *P = (T *)ws(WS_T3, (size_t)(chunks * m) * sizeof(T));
  if (!P) return MATGB_ERR_NOMEM;
  if (n > 0) {
    gemv_partial_kernel<T><<<dim3((unsigned)rb, (unsigned)chunks), kGemvRows, 0,
                          c->stream>>>(m, n, cols_per, A, lda, x, P);
    MGB_LAUNCHED("gemv_partial");
  } else {
    MGB_CUDA(cudaMemsetAsync(P, 0, (size_t)m * sizeof(T), c->stream));
  }
  gemv_reduce_kernel<T><<<(unsigned)((m + 255) / 256), 256, 0, c->stream>>>(
      m, (int)chunks, alpha, P, beta, y);
  MGB_LAUNCHED("gemv_reduce");
  return 0;
}
template int gemv_t<float>(int64_t, int64_t, float, const float *, int64_t,
                           const float *, float, float *);
template int gemv_t<double>(int64_t, int64_t, double, const double *, int64_t,
                            const double *, double, double *);

int gemv(int64_t m, int64_t n, elem_t alpha, const elem_t *A, int64_t lda,
         const elem_t *x, elem_t beta, elem_t *y) {
  return gemv_t<elem_t>(m, n, alpha, A, lda, x, beta, y);
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_gemm_dev(char transa, char transb, size_t m, size_t n, size_t k,
                   mat_elem_t alpha, const mat_elem_t *A, size_t lda,
                   const mat_elem_t *B, size_t ldb, mat_elem_t beta,
                   mat_elem_t *C, size_t ldc) {
  bool ta = (transa == 'T' || transa == 't');
  bool tb = (transb == 'T' || transb == 't');
  if ((!ta && transa != 'N' && transa != 'n') ||
      (!tb && transb != 'N' && transb != 'n'))
    return set_error(MATGB_ERR_ARG, "gemm: trans flags must be N or T");
  if (ldc < m || lda < (ta ? k : m) || ldb < (tb ? n : k))
    return set_error(MATGB_ERR_ARG, "gemm: leading dimension too small");
  return gemm(ta, tb, (int64_t)m, (int64_t)n, (int64_t)k, alpha, A,
              (int64_t)lda, B, (int64_t)ldb, beta, C, (int64_t)ldc, 0);
}

int matgb_syrk_dev(char uplo, char trans, size_t n, size_t k, mat_elem_t alpha,
                   const mat_elem_t *A, size_t lda, mat_elem_t beta,
                   mat_elem_t *C, size_t ldc) {
  int tri = (uplo == 'L' || uplo == 'l') ? 1 : (uplo == 'U' || uplo == 'u') ? 2 : 0;
  bool t = (trans == 'T' || trans == 't');
  if (!tri || (!t && trans != 'N' && trans != 'n'))
    return set_error(MATGB_ERR_ARG, "syrk: bad uplo/trans");
  if (ldc < n || lda < (t ? k : n))
    return set_error(MATGB_ERR_ARG, "syrk: leading dimension too small");
  // 'N': C = alpha*A*A^T (A n x k);  'T': C = alpha*A^T*A (A k x n).
  return gemm(t, !t, (int64_t)n, (int64_t)n, (int64_t)k, alpha, A,
              (int64_t)lda, A, (int64_t)lda, beta, C, (int64_t)ldc, tri);
}

int matgb_gemv_dev(size_t m, size_t n, mat_elem_t alpha, const mat_elem_t *A,
                   size_t lda, const mat_elem_t *x, mat_elem_t beta,
                   mat_elem_t *y) {
  if (lda < m) return set_error(MATGB_ERR_ARG, "gemv: lda < m");
  return gemv((int64_t)m, (int64_t)n, alpha, A, (int64_t)lda, x, beta, y);
}

}  // extern "C"

// ---- GEMV without allocation -------------------------------------------------
// For callers that must not allocate device memory: the column-split partial
// sums live in this file-scope device array instead of the library's
// workspace, and the caller supplies the stream.  Every GPU that loads the
// library holds the array (kGemvStaticElems elements: 4 MiB in libmatgb_f32,
// 8 MiB in libmatgb_f64) until the process exits.
#include <mutex>

namespace mgb {

constexpr size_t kGemvStaticElems = (size_t)1 << 20;
static __device__ __align__(256) elem_t g_gemv_static_scratch[kGemvStaticElems];

// Device address of the array for the current device, looked up once per
// device (host code may not use the symbol's host-side name as a pointer).
static int gemv_static_scratch(elem_t **out, int *sms) {
  static std::mutex mu;
  static elem_t *addr[64] = {};
  static int nsm[64] = {};
  int dev = -1;
  MGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(MATGB_ERR_ARG, "device id %d", dev);
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    MGB_CUDA(cudaGetSymbolAddress(&p, g_gemv_static_scratch));
    MGB_CUDA(cudaDeviceGetAttribute(&nsm[dev], cudaDevAttrMultiProcessorCount, dev));
    addr[dev] = (elem_t *)p;
  }
  *out = addr[dev];
  *sms = nsm[dev];
  return 0;
}

}  // namespace mgb

extern "C" int matgb_gemv_noalloc_dev(size_t m, size_t n, mat_elem_t alpha,
                                      const mat_elem_t *A, size_t lda,
                                      const mat_elem_t *x, mat_elem_t beta,
                                      mat_elem_t *y, void *stream) {
  using namespace mgb;
  if (lda < m) return set_error(MATGB_ERR_ARG, "gemv_noalloc: lda < m");
  if (m > kGemvStaticElems)
    return set_error(MATGB_ERR_ARG,
                     "gemv_noalloc: m = %zu exceeds the static scratch of %zu "
                     "elements",
                     m, kGemvStaticElems);
  if (m == 0) return 0;
  elem_t *P = nullptr;
  int sms = 0;
  MGB_TRY(gemv_static_scratch(&P, &sms));
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t M = (int64_t)m, N = (int64_t)n;
  const int64_t rb = (M + kGemvRows - 1) / kGemvRows;
  const int64_t target = (int64_t)(sms > 0 ? sms : 148) * 8;
  int64_t chunks = (target + rb - 1) / rb;
  const int64_t cap = (int64_t)(kGemvStaticElems / m);
  if (chunks > cap) chunks = cap;
  if (chunks > N) chunks = N;
  if (chunks > 1024) chunks = 1024;
  int64_t cols_per = 0;
  if (N > 0) {
    if (chunks < 1) chunks = 1;
    cols_per = (N + chunks - 1) / chunks;
    chunks = (N + cols_per - 1) / cols_per;
    // every (chunk, row) slot read below is written here first, so the
    // array needs no clearing between calls
    gemv_partial_kernel<elem_t><<<dim3((unsigned)rb, (unsigned)chunks),
                                  kGemvRows, 0, st>>>(M, N, cols_per, A,
                                                      (int64_t)lda, x, P);
    MGB_LAUNCHED("gemv_partial_noalloc");
  } else {
    chunks = 0;  // y = beta*y; nothing is read from the array
  }
  gemv_reduce_kernel<elem_t><<<(unsigned)((M + 255) / 256), 256, 0, st>>>(
      M, (int)chunks, alpha, P, beta, y);
  MGB_LAUNCHED("gemv_reduce_noalloc");
  return 0;
}
