// Lower Cholesky (mat_chol / mat_solve_spd's factorisation).
//
// Reference: mat_chol (mat.h:6062-6092) factors the lower triangle and returns
// -1 at the first diagonal that is <= 0 (mat.h:5973-5975, 6046-6048); its
// blocked NEON path (mat__chol_blocked_, mat.h:5988-6027) is panel potrf ->
// TRSM (L21 = A21 L11^-T by axpy/scal with the reciprocal of L_jj) -> SYRK
// trailing update (mat__syrk_lower_, k = block, alpha = -1, beta = 1).
//
// GB300: blocks of 96.  The diagonal block is factored by one CTA in shared
// memory; the panel TRSM is one kernel over 32-row tiles (L11 and the rows in
// shared memory); the trailing update is the lower-triangle-masked GEMM.
// Every kernel returns at once when *info != 0 so a failure stops the chain
// without a host round trip.
#include "internal.cuh"

namespace mgb {

constexpr int kCholBlock = 96;

static size_t diag_smem(int nb) { return (size_t)nb * (nb + 1) * sizeof(elem_t); }
static size_t ctrsm_smem(int nb) {
  return ((size_t)nb * (nb + 1) + (size_t)nb * 33) * sizeof(elem_t);
}

__global__ void __launch_bounds__(256)
    potrf_diag_kernel(int nb, elem_t *__restrict__ A, int64_t lda,
                      int32_t *__restrict__ info, int64_t kb) {
  if (*info != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  elem_t *Ls = (elem_t *)smem_raw;  // Ls[j*(nb+1)+i]
  const int tid = threadIdx.x;
  const int ld = nb + 1;
  for (int e = tid; e < nb * nb; e += 256) {
    int i = e % nb, j = e / nb;
    Ls[j * ld + i] = (i >= j) ? A[i + (int64_t)j * lda] : elem_t(0);
  }
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    const elem_t d = Ls[j * ld + j];
    if (d <= 0) {  // NaN passes, as in the reference's "diag <= 0" test
      if (tid == 0) *info = (int32_t)(kb + j + 1);
      break;
    }
    const elem_t ljj = sqrt(d);
    const elem_t inv = elem_t(1) / ljj;
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
__global__ void __launch_bounds__(256)
    chol_trsm_kernel(int nb, const elem_t *__restrict__ L11, elem_t *__restrict__ A21,
                     int64_t lda, int64_t m, const int32_t *__restrict__ info) {
  if (*info != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  elem_t *Ls = (elem_t *)smem_raw;              // Ls[j*(nb+1)+i] = L11(i,j)
  elem_t *Xs = Ls + (size_t)nb * (nb + 1);      // Xs[j*33 + rr]
  const int tid = threadIdx.x, rr = tid & 31, g = tid >> 5;
  const int ld = nb + 1;
  const int64_t r0 = (int64_t)blockIdx.x * 32;
  for (int e = tid; e < nb * nb; e += 256) {
    int i = e % nb, j = e / nb;
    Ls[j * ld + i] = L11[i + (int64_t)j * lda];
  }
  for (int e = tid; e < nb * 32; e += 256) {
    int r = e % 32, j = e / 32;
    Xs[j * 33 + r] = (r0 + r < m) ? A21[(r0 + r) + (int64_t)j * lda] : elem_t(0);
  }
  __syncthreads();
  if (g == 0) Xs[rr] = Xs[rr] * (elem_t(1) / Ls[0]);
  __syncthreads();
  for (int j = 0; j < nb; j++) {
    const elem_t xj = Xs[j * 33 + rr];
    for (int k = j + 1 + g; k < nb; k += 8) {
      elem_t v = fma(-xj, Ls[j * ld + k], Xs[k * 33 + rr]);
      if (k == j + 1) v = v * (elem_t(1) / Ls[k * ld + k]);
      Xs[k * 33 + rr] = v;
    }
    __syncthreads();
  }
  for (int e = tid; e < nb * 32; e += 256) {
    int r = e % 32, j = e / 32;
    if (r0 + r < m) A21[(r0 + r) + (int64_t)j * lda] = Xs[j * 33 + r];
  }
}

static bool g_chol_ready = false;

int potrf(int64_t n, elem_t *A, int64_t lda, int32_t *info) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  MGB_CUDA(cudaMemsetAsync(info, 0, sizeof(int32_t), cx->stream));
  if (n <= 0) return 0;
  if (!g_chol_ready) {
    MGB_CUDA(cudaFuncSetAttribute(potrf_diag_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)diag_smem(kCholBlock)));
    MGB_CUDA(cudaFuncSetAttribute(chol_trsm_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)ctrsm_smem(kCholBlock)));
    g_chol_ready = true;
  }
  for (int64_t kb = 0; kb < n; kb += kCholBlock) {
    const int nb = (int)((n - kb) < kCholBlock ? (n - kb) : kCholBlock);
    elem_t *A11 = A + kb + kb * lda;
    KtScope kt("potrf_diag", nb * (double)nb * nb / 3.0,
               (double)nb * nb * sizeof(elem_t));
    potrf_diag_kernel<<<1, 256, diag_smem(nb), cx->stream>>>(nb, A11, lda, info,
                                                             kb);
    MGB_LAUNCHED("potrf_diag");
    const int64_t m = n - kb - nb;
    if (m > 0) {
      elem_t *A21 = A + (kb + nb) + kb * lda;
      KtScope kt2("chol_trsm", (double)m * nb * nb,
                  2.0 * m * nb * sizeof(elem_t));
      chol_trsm_kernel<<<(unsigned)((m + 31) / 32), 256, ctrsm_smem(nb),
                         cx->stream>>>(nb, A11, A21, lda, m, info);
      MGB_LAUNCHED("chol_trsm");
      MGB_TRY(gemm_skip(false, true, m, m, nb, elem_t(-1), A21, lda, A21, lda,
                        elem_t(1), A + (kb + nb) + (kb + nb) * lda, lda, 1,
                        info));
    }
  }
  return 0;
}

int potrs(int64_t n, int64_t nrhs, const elem_t *L, int64_t lda, elem_t *B,
          int64_t ldb, const int32_t *info) {
  MGB_TRY(trsm_left(true, false, false, n, nrhs, L, lda, B, ldb, info));
  MGB_TRY(trsm_left(true, true, false, n, nrhs, L, lda, B, ldb, info));
  return 0;
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

}  // extern "C"
