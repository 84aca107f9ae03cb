// Lower Cholesky (mat_chol / mat_solve_spd's factorisation).
//
// Reference: mat_chol (mat.h:6062-6092) factors the lower triangle and returns
// -1 at the first diagonal that is <= 0 (mat.h:5973-5975, 6046-6048); its
// blocked NEON path (mat__chol_blocked_, mat.h:5988-6027) is panel potrf ->
// TRSM (L21 = A21 L11^-T by axpy/scal with the reciprocal of L_jj) -> SYRK
// trailing update (mat__syrk_lower_, k = block, alpha = -1, beta = 1).
//
// GB300: blocks of 96 (128 on the tensor-core path).  The diagonal block is
// factored by one CTA in shared memory; the panel TRSM is one kernel over
// 32-row tiles (L11 and the rows in shared memory); the trailing update is the
// lower-triangle-masked SIMT GEMM, or for the mixed-precision solver the
// tensor-core rank-K update with L21 packed once to BF16/FP16 (FP16 with a
// power-of-two scale) and used as both operands, lower tiles only.  Every
// kernel returns at once when *info != 0 so a failure stops the chain without
// a host round trip.
#include "internal.cuh"

namespace mgb {

constexpr int kCholBlock = 96;
constexpr int kCholBlockLp = 128;

template <typename T>
static size_t diag_smem(int nb) { return (size_t)nb * (nb + 1) * sizeof(T); }
template <typename T>
static size_t ctrsm_smem(int nb) {
  return ((size_t)nb * (nb + 1) + (size_t)nb * 33) * sizeof(T);
}

template <typename T>
__global__ void __launch_bounds__(256)
    potrf_diag_kernel(int nb, T *__restrict__ A, int64_t lda,
                      int32_t *__restrict__ info, int64_t kb) {
  if (*info != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *Ls = (T *)smem_raw;  // Ls[j*(nb+1)+i]
  const int tid = threadIdx.x;
  const int ld = nb + 1;
  for (int e = tid; e < nb * nb; e += 256) {
    int i = e % nb, j = e / nb;
    Ls[j * ld + i] = (i >= j) ? A[i + (int64_t)j * lda] : T(0);
  }
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    const T d = Ls[j * ld + j];
    if (d <= 0) {  // NaN passes, as in the reference's "diag <= 0" test
      if (tid == 0) *info = (int32_t)(kb + j + 1);
      break;
    }
    const T ljj = sqrt(d);
    const T inv = T(1) / ljj;
    __syncthreads();  // everyone has read d
    if (tid == 0) Ls[j * ld + j] = ljj;
    for (int i = j + 1 + tid; i < nb; i += 256) Ls[j * ld + i] *= inv;
    __syncthreads();
    const int r = nb - j - 1;
    for (int e = tid; e < r * r; e += 256) {
      const int i = j + 1 + e % r, k = j + 1 + e / r;
      if (k <= i) Ls[k * ld + i] = fma(-Ls[j * ld + i], Ls[j * ld + k], Ls[k * ld + i]);
    }
    __syncthreads();
  }
  __syncthreads();
  for (int e = tid; e < nb * nb; e += 256) {
    int i = e % nb, j = e / nb;
    if (i >= j) A[i + (int64_t)j * lda] = Ls[j * ld + i];
  }
}

// L21 (m x nb, rows of A below the diagonal block) <- A21 * L11^{-T}.
// CTA: 32 rows; thread (row rr = tid%32, group g = tid/32) updates columns
// k = j+1+g, j+9+g, ... after column j is final.
template <typename T>
__global__ void __launch_bounds__(256)
    chol_trsm_kernel(int nb, const T *__restrict__ L11, T *__restrict__ A21,
                     int64_t lda, int64_t m, const int32_t *__restrict__ info) {
  if (*info != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *Ls = (T *)smem_raw;                   // Ls[j*(nb+1)+i] = L11(i,j)
  T *Xs = Ls + (size_t)nb * (nb + 1);      // Xs[j*33 + rr]
  const int tid = threadIdx.x, rr = tid & 31, g = tid >> 5;
  const int ld = nb + 1;
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  for (int e = tid; e < nb * nb; e += 256) {
    int i = e % nb, j = e / nb;
    Ls[j * ld + i] = L11[i + (int64_t)j * lda];
  }
  for (int e = tid; e < nb * 32; e += 256) {
    int r = e % 32, j = e / 32;
    Xs[j * 33 + r] = (r0 + r < m) ? A21[(r0 + r) + (int64_t)j * lda] : T(0);
  }
  __syncthreads();
  if (g == 0) Xs[rr] = Xs[rr] * (T(1) / Ls[0]);
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    const T xj = Xs[j * 33 + rr];
    for (int k = j + 1 + g; k < nb; k += 8) {
      T v = fma(-xj, Ls[j * ld + k], Xs[k * 33 + rr]);
      if (k == j + 1) v = v * (T(1) / Ls[k * ld + k]);
      Xs[k * 33 + rr] = v;
    }
    __syncthreads();
  }
  for (int e = tid; e < nb * 32; e += 256) {
    int r = e % 32, j = e / 32;
    if (r0 + r < m) A21[(r0 + r) + (int64_t)j * lda] = Xs[j * 33 + r];
  }
}

template <typename T>
int potrf_t(int64_t n, T *A, int64_t lda, int32_t *info, int lp) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  MGB_CUDA(cudaMemsetAsync(info, 0, sizeof(int32_t), cx->stream));
  if (n <= 0) return 0;
  if (lp >= 0 && sizeof(T) != 4)
    return set_error(MATGB_ERR_ARG, "tensor-core Cholesky is float");
  const int NB = lp >= 0 ? kCholBlockLp : kCholBlock;
  // the shared-memory opt-in is set on every call (a host-side attribute
  // write), through the same function pointers the launches use
  auto kdiag = potrf_diag_kernel<T>;
  auto ktrsm = chol_trsm_kernel<T>;
  MGB_CUDA(cudaFuncSetAttribute(kdiag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)diag_smem<T>(NB)));
  MGB_CUDA(cudaFuncSetAttribute(ktrsm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)ctrsm_smem<T>(NB)));
  for (int64_t kb = 0; kb < n; kb += NB) {
    const int nb = (int)((n - kb) < NB ? (n - kb) : NB);
    T *A11 = A + kb + kb * lda;
    {
      KtScope kt("potrf_diag", nb * (double)nb * nb / 3.0,
                 (double)nb * nb * sizeof(T));
      kdiag<<<1, 256, diag_smem<T>(nb), cx->stream>>>(nb, A11, lda, info, kb);
      MGB_TRY(launch_check((const void *)kdiag, "potrf_diag", diag_smem<T>(nb)));
    }
    const int64_t m = n - kb - nb;
    if (m > 0) {
      T *A21 = A + (kb + nb) + kb * lda;
      {
        KtScope kt2("chol_trsm", (double)m * nb * nb,
                    2.0 * m * nb * sizeof(T));
        ktrsm<<<(unsigned)((m + 31) / 32), 256, ctrsm_smem<T>(nb), cx->stream>>>(
            nb, A11, A21, lda, m, info);
        MGB_TRY(launch_check((const void *)ktrsm, "chol_trsm", ctrsm_smem<T>(nb)));
      }
      T *A22 = A + (kb + nb) + (kb + nb) * lda;
      if (lp < 0)
        MGB_TRY(gemm_skip_t<T>(false, true, m, m, nb, T(-1), A21, lda, A21, lda,
                               T(1), A22, lda, 1, info));
      else
        MGB_TRY(lp_syrk_update(m, nb, (float *)A21, lda, (float *)A22, lda, lp,
                               info));
    }
  }
  return 0;
}

template <typename T>
int potrs_t(int64_t n, int64_t nrhs, const T *L, int64_t lda, T *B,
            int64_t ldb, const int32_t *info) {
  MGB_TRY(trsm_left_t<T>(true, false, false, n, nrhs, L, lda, B, ldb, info));
  MGB_TRY(trsm_left_t<T>(true, true, false, n, nrhs, L, lda, B, ldb, info));
  return 0;
}

template int potrf_t<float>(int64_t, float *, int64_t, int32_t *, int);
template int potrf_t<double>(int64_t, double *, int64_t, int32_t *, int);
template int potrs_t<float>(int64_t, int64_t, const float *, int64_t, float *,
                            int64_t, const int32_t *);
template int potrs_t<double>(int64_t, int64_t, const double *, int64_t,
                             double *, int64_t, const int32_t *);

int potrf(int64_t n, elem_t *A, int64_t lda, int32_t *info) {
  return potrf_t<elem_t>(n, A, lda, info, -1);
}

int potrs(int64_t n, int64_t nrhs, const elem_t *L, int64_t lda, elem_t *B,
          int64_t ldb, const int32_t *info) {
  return potrs_t<elem_t>(n, nrhs, L, lda, B, ldb, info);
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_potrf_dev(size_t n, mat_elem_t *A, size_t lda, int32_t *info) {
  if (lda < n) return set_error(MATGB_ERR_ARG, "potrf: lda < n");
  if (!info) return set_error(MATGB_ERR_ARG, "potrf: info is NULL");
  return potrf((int64_t)n, A, (int64_t)lda, info);
}

int matgb_potrs_dev(size_t n, size_t nrhs, const mat_elem_t *L, size_t lda,
                    mat_elem_t *B, size_t ldb, const int32_t *info) {
  if (lda < n || ldb < n)
    return set_error(MATGB_ERR_ARG, "potrs: leading dimension too small");
  return potrs((int64_t)n, (int64_t)nrhs, L, (int64_t)lda, B, (int64_t)ldb,
               info);
}

int matgb_potrf_lp_dev(size_t n, float *A, size_t lda, int32_t *info,
                       int lp_format) {
  if (lda < n) return set_error(MATGB_ERR_ARG, "potrf_lp: lda < n");
  if (!info) return set_error(MATGB_ERR_ARG, "potrf_lp: info is NULL");
  if (lp_format < -1 || lp_format > 2)
    return set_error(MATGB_ERR_ARG, "potrf_lp: lp_format");
  return potrf_t<float>((int64_t)n, A, (int64_t)lda, info, lp_format);
}

}  // extern "C"
