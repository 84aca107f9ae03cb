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
static size_t rows_smem(int NB) { return ((size_t)NB * (NB + 4) + NB) * sizeof(float); }
template <typename T>
static size_t ctrsm_smem(int nb) {
  return ((size_t)nb * (nb + 1) + (size_t)nb * 33) * sizeof(T);
}

constexpr int kDiagMax = 128;  // largest diagonal block (kCholBlock, kCholBlockLp)

template <typename T>
__global__ void __launch_bounds__(256)
    potrf_diag_kernel(int nb, T *__restrict__ A, int64_t lda,
                      int32_t *__restrict__ info, int64_t kb) {
  if (*info != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *Ls = (T *)smem_raw;  // Ls[j*(nb+1)+i] = A(i, j), lower triangle only
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int ld = nb + 1;
  for (int j = ty; j < nb; j += 16)
    for (int i = j + tx; i < nb; i += 16) Ls[j * ld + i] = A[i + (int64_t)j * lda];
  __syncthreads();
  // Column j: d = A(j,j), L(j,j) = sqrt(d), L(i,j) = A(i,j) * (1/L(j,j)) and
  // the trailing lower triangle A(i,k) -= L(i,j) L(k,j).  Threads: 16 x 16
  // over (row, column) of the trailing triangle, no divisions.
  // the scaled column in its own array, so the update's reads never alias
  // its writes and the loads pipeline
  __shared__ T colj[kDiagMax];
  for (int j = 0; j < nb; j++) {
    const T d = Ls[j * ld + j];
    if (d <= T(0)) {  // NaN passes, as in the reference's "diag <= 0" test
      if (tid == 0) *info = (int32_t)(kb + j + 1);
      break;
    }
    const T ljj = sqrt(d);
    const T inv = T(1) / ljj;
    for (int i = j + 1 + tid; i < nb; i += 256) {
      const T l = Ls[j * ld + i] * inv;
      colj[i] = l;
      Ls[j * ld + i] = l;
    }
    __syncthreads();
    if (tid == 0) Ls[j * ld + j] = ljj;
    for (int k = j + 1 + ty; k < nb; k += 16) {
      const T lkj = colj[k];
      for (int i = k + tx; i < nb; i += 16) Ls[k * ld + i] = fma(-colj[i], lkj, Ls[k * ld + i]);
    }
    __syncthreads();
  }
  __syncthreads();
  for (int j = ty; j < nb; j += 16)
    for (int i = j + tx; i < nb; i += 16) A[i + (int64_t)j * lda] = Ls[j * ld + i];
}

// Float form, one thread per row of the diagonal block (NB threads): before
// step j row i >= j holds A^(j)(i, j..i) in a[0..i-j] (shifted frame).  Step
// j: every row publishes a[0] (column j; the pivot d at its head) into a
// double-buffered shared column, one barrier, then L(j,j) = sqrt(d), row i
// writes L(i,j) = a[0] * (1/L(j,j)) and updates A(i,k) -= L(i,j) L(k,j),
// forming each L(k,j) from the published column the same way -- the
// operands and FMAs of potrf_diag_kernel, with one barrier per column.
template <int NB>
__global__ void __launch_bounds__(NB)
    potrf_diag_rows_kernel(int nb, float *__restrict__ A, int64_t lda,
                           int32_t *__restrict__ info, int64_t kb,
                           unsigned *__restrict__ zero = nullptr) {
  // zero (may be null): the max slot that the column solve after this
  // kernel fills, cleared here instead of by a launch of its own
  if (zero && threadIdx.x == 0) *zero = 0u;
  if (*info != 0) return;
  __shared__ __align__(16) float colb[2][NB + 8];  // colb[.][3 + (i - j)] = A^(j)(i, j)
  const int i = threadIdx.x;
  const bool act = i < nb;
  const int wlast = ((i | 31) < nb - 1 ? (i | 31) : nb - 1);  // the warp's last row
  float a[NB];
#pragma unroll
  for (int c = 0; c < NB; c++) a[c] = (act && c <= i) ? A[i + (int64_t)c * lda] : 0.f;
  for (int j = 0; j < nb; j++) {
    float *cb = colb[j & 1];
    if (act && i >= j) cb[3 + (i - j)] = a[0];
    __syncthreads();
    const float d = cb[3];
    if (d <= 0.f) {  // NaN passes, as in the reference's "diag <= 0" test
      if (i == 0) *info = (int32_t)(kb + j + 1);
      return;
    }
    const float ljj = sqrtf(d);
    const float inv = 1.f / ljj;
    if (act && i >= j) A[i + (int64_t)j * lda] = i == j ? ljj : a[0] * inv;
    const int n_out = wlast - j;  // the warp's longest remaining row
    if (n_out > 0) {
      const float lij = a[0] * inv;
      const bool upd = act && i > j;
#pragma unroll
      for (int c = 0; c < NB / 32; c++) {
        if (c * 32 < n_out) {
#pragma unroll
          for (int k0 = c * 32; k0 < c * 32 + 32; k0 += 4) {
            const float4 u = *reinterpret_cast<const float4 *>(cb + 4 + k0);
            const float uu[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int q = 0; q < 4; q++)
              if (k0 + q + 1 < NB)
                a[k0 + q] = upd ? fma(-lij, uu[q] * inv, a[k0 + q + 1]) : a[k0 + q + 1];
          }
        }
      }
    }
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

// Float form of the same solve, one thread per row of L21 (128 rows per CTA):
// row r is independent of the others, x_j = (a_j - sum_{k<j} x_k L(j,k)) /
// L(j,j).  The row sits in registers in a shifted frame (before step j,
// a[0..] are its pending columns j, j+1, ...), so the column loop is an
// ordinary loop over static register indices; step j's column of L11 below
// the diagonal is read from shared memory with 16-byte broadcast loads.
// The same FMAs on the same operands as chol_trsm_kernel, in the same order,
// and no block barrier inside the solve.
template <int NB>
__global__ void __launch_bounds__(128)
    chol_trsm_rows_kernel(int nb, const float *__restrict__ L11, float *__restrict__ A21,
                          int64_t lda, int64_t m, const int32_t *__restrict__ info,
                          unsigned *__restrict__ amax = nullptr) {
  if (*info != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float (*Lt)[NB + 4] = reinterpret_cast<float (*)[NB + 4]>(smem_raw);  // Lt[j][k] = L11(j+1+k, j)
  float *rinv = reinterpret_cast<float *>(smem_raw) + (size_t)NB * (NB + 4);
  const int tid = threadIdx.x;
  for (int j = 0; j < nb; j++)
    for (int k = tid; k < NB; k += 128)
      Lt[j][k] = (j + 1 + k < nb) ? L11[(j + 1 + k) + (int64_t)j * lda] : 0.f;
  for (int j = tid; j < nb; j += 128) rinv[j] = 1.f / L11[j + (int64_t)j * lda];
  __syncthreads();
  const int64_t r = (int64_t)blockIdx.x * 128 + tid;
  const bool act = r < m;
  float a[NB];
#pragma unroll
  for (int j = 0; j < NB; j++) a[j] = (act && j < nb) ? A21[r + (int64_t)j * lda] : 0.f;
  float mx = 0.f;  // max |L21| over the row (amax given); NaN ignored as in amax_kernel
  for (int j = 0; j < nb; j++) {
    const float x = a[0] * rinv[j];
    if (act) A21[r + (int64_t)j * lda] = x;
    if (act) mx = fmaxf(mx, fabsf(x));
    const int n_out = nb - 1 - j;  // pending columns after this step
#pragma unroll
    for (int c = 0; c < NB / 32; c++) {
      if (c * 32 < n_out) {
#pragma unroll
        for (int k0 = c * 32; k0 < c * 32 + 32; k0 += 4) {
          const float4 u = *reinterpret_cast<const float4 *>(&Lt[j][k0]);
          const float uu[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
          for (int q = 0; q < 4; q++)
            if (k0 + q + 1 < NB) a[k0 + q] = fma(-x, uu[q], a[k0 + q + 1]);
        }
      }
    }
  }
  if (amax) {
    for (int off = 16; off; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if ((tid & 31) == 0) atomicMax(amax, __float_as_uint(mx));
  }
}

// The diagonal block [kb, kb+nb) and the column solve below it, on the
// current library stream.
// amax (may be null): for a float block of 96 or 128 columns the kernels
// also leave max |L21| there (zeroed by the diagonal kernel); *amax_done
// says whether they did.
template <typename T>
static int chol_panel(int64_t n, T *A, int64_t lda, int32_t *info, int64_t kb, int nb,
                      unsigned *amax = nullptr, bool *amax_done = nullptr) {
  if (amax_done) *amax_done = false;
  Ctx *cx = ctx();
  T *A11 = A + kb + kb * lda;
  {
    KtScope kt("potrf_diag", nb * (double)nb * nb / 3.0,
               (double)nb * nb * sizeof(T));
    if (sizeof(T) == 4 && nb > 64) {
      if (nb > kCholBlock) {
        potrf_diag_rows_kernel<kCholBlockLp><<<1, kCholBlockLp, 0, cx->stream>>>(
            nb, (float *)A11, lda, info, kb, amax);
        MGB_TRY(launch_check((const void *)potrf_diag_rows_kernel<kCholBlockLp>,
                             "potrf_diag_rows", 0));
      } else {
        potrf_diag_rows_kernel<kCholBlock><<<1, kCholBlock, 0, cx->stream>>>(
            nb, (float *)A11, lda, info, kb, amax);
        MGB_TRY(launch_check((const void *)potrf_diag_rows_kernel<kCholBlock>,
                             "potrf_diag_rows", 0));
      }
    } else {
      auto kdiag = potrf_diag_kernel<T>;
      kdiag<<<1, 256, diag_smem<T>(nb), cx->stream>>>(nb, A11, lda, info, kb);
      MGB_TRY(launch_check((const void *)kdiag, "potrf_diag", diag_smem<T>(nb)));
    }
  }
  const int64_t m = n - kb - nb;
  if (m <= 0) return 0;
  T *A21 = A + (kb + nb) + kb * lda;
  KtScope kt2("chol_trsm", (double)m * nb * nb, 2.0 * m * nb * sizeof(T));
  if constexpr (sizeof(T) == 4) {
    if (nb == kCholBlockLp || nb == kCholBlock) {
      const size_t sm = nb == kCholBlockLp ? rows_smem(kCholBlockLp) : rows_smem(kCholBlock);
      const void *kr = nb == kCholBlockLp ? (const void *)chol_trsm_rows_kernel<kCholBlockLp>
                                          : (const void *)chol_trsm_rows_kernel<kCholBlock>;
      MGB_CUDA(cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      if (nb == kCholBlockLp)
        chol_trsm_rows_kernel<kCholBlockLp><<<(unsigned)((m + 127) / 128), 128, sm, cx->stream>>>(
            nb, (const float *)A11, (float *)A21, lda, m, info, amax);
      else
        chol_trsm_rows_kernel<kCholBlock><<<(unsigned)((m + 127) / 128), 128, sm, cx->stream>>>(
            nb, (const float *)A11, (float *)A21, lda, m, info, amax);
      MGB_TRY(launch_check(kr, "chol_trsm_rows", sm));
      // both kernels ran in their row forms (nb > 64): the max is there
      if (amax_done) *amax_done = amax != nullptr && nb > 64;
      return 0;
    }
  }
  auto ktrsm = chol_trsm_kernel<T>;
  ktrsm<<<(unsigned)((m + 31) / 32), 256, ctrsm_smem<T>(nb), cx->stream>>>(nb, A11, A21, lda,
                                                                         m, info);
  return launch_check((const void *)ktrsm, "chol_trsm", ctrsm_smem<T>(nb));
}

// Look-ahead for the tensor-core Cholesky (float, lp >= 0).  The panel chain
// runs on a high-priority stream: block k's diagonal factor, its column
// solve, its L21 packed (buffer set k % 2), then the next block's columns
// updated with it; the library stream updates the rest of the trailing
// matrix with the same packed operand meanwhile.  The next block's columns
// are also written by the previous block's rest update, so the panel stream
// waits for that one (evr) before its own update of them; the rest update
// waits for the packing (evp).  A packing buffer is rewritten two blocks
// later, after the panel stream has waited for the rest update that read it.
struct CholLookAhead {
  cudaStream_t hi = nullptr;
  cudaEvent_t ev0 = nullptr, evp = nullptr, evr = nullptr, evend = nullptr;
  bool ready = false;
};
static CholLookAhead g_cla;
static int g_chol_la = 1;

static int chol_la_setup() {
  if (g_cla.ready) return 0;
  int lo = 0, hi = 0;
  MGB_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  MGB_CUDA(cudaStreamCreateWithPriority(&g_cla.hi, cudaStreamNonBlocking, hi));
  for (cudaEvent_t *e : {&g_cla.ev0, &g_cla.evp, &g_cla.evr, &g_cla.evend})
    MGB_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  g_cla.ready = true;
  return 0;
}

static int potrf_la(int64_t n, float *A, int64_t lda, int32_t *info, int lp) {
  MGB_TRY(chol_la_setup());
  const int NB = kCholBlockLp;
  cudaStream_t main = ctx()->stream, hi = g_cla.hi;
  if (n > NB) {
    // both packing sets at their largest (block 0's) size, grown here while
    // the library stream is current (a growth waits for its users first)
    const size_t bytes = (size_t)(n - NB) * ((NB + 63) / 64 * 64) * 2 * (lp == 2 ? 2 : 1);
    if (!ws(WS_T0, bytes) || !ws(WS_CU0, bytes) || !ws(WS_T2, 64) || !ws(WS_CU0 + 2, 64))
      return MATGB_ERR_NOMEM;
  }
  MGB_CUDA(cudaEventRecord(g_cla.ev0, main));
  MGB_CUDA(cudaStreamWaitEvent(hi, g_cla.ev0, 0));
  MGB_CUDA(cudaEventRecord(g_cla.evr, main));
  for (int64_t kb = 0, k = 0; kb < n; kb += NB, k++) {
    const int nb = (int)((n - kb) < NB ? (n - kb) : NB);
    const int64_t m = n - kb - nb;
    const int64_t nn = m < NB ? m : NB;  // the next block's width
    float *A21 = A + (kb + nb) + kb * lda;
    SyrkOperand op{};
    {
      StreamSwap sw(hi);
      // the FP16 scale's max comes from the block's own kernels
      unsigned *slot = (m > 0 && lp != 1) ? lp_syrk_amax_slot((int)(k & 1)) : nullptr;
      bool amax_done = false;
      MGB_TRY(chol_panel<float>(n, A, lda, info, kb, nb, slot, &amax_done));
      if (m > 0) {
        // (set k % 2 was last read by block k-2's rest update, which the
        // panel stream waited for before block k-1's look-ahead update)
        MGB_TRY(lp_syrk_pack(m, nb, A21, lda, lp, (int)(k & 1), &op, amax_done));
        MGB_CUDA(cudaEventRecord(g_cla.evp, hi));
        MGB_CUDA(cudaStreamWaitEvent(hi, g_cla.evr, 0));
        MGB_TRY(lp_syrk_apply(op, 0, m, 0, nn, A + (kb + nb) + (kb + nb) * lda, lda, info));
      }
    }
    if (m > nn) {
      // one CTA per tile: the persistent form would hold every SM for the
      // whole update and starve the panel chain beside it
      MGB_CUDA(cudaStreamWaitEvent(main, g_cla.evp, 0));
      MGB_TRY(lp_syrk_apply(op, nn, m - nn, nn, m - nn,
                            A + (kb + nb + nn) + (kb + nb + nn) * lda, lda, info, 0));
      MGB_CUDA(cudaEventRecord(g_cla.evr, main));
    }
  }
  // the library stream resumes after the panel stream's last work
  MGB_CUDA(cudaEventRecord(g_cla.evend, hi));
  MGB_CUDA(cudaStreamWaitEvent(main, g_cla.evend, 0));
  return 0;
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
  MGB_CUDA(cudaFuncSetAttribute(potrf_diag_kernel<T>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)diag_smem<T>(NB)));
  MGB_CUDA(cudaFuncSetAttribute(chol_trsm_kernel<T>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)ctrsm_smem<T>(NB)));
  if constexpr (sizeof(T) == 4) {
    if (lp >= 0 && g_chol_la) return potrf_la(n, (float *)A, lda, info, lp);
  }
  for (int64_t kb = 0; kb < n; kb += NB) {
    const int nb = (int)((n - kb) < NB ? (n - kb) : NB);
    MGB_TRY(chol_panel<T>(n, A, lda, info, kb, nb));
    const int64_t m = n - kb - nb;
    if (m > 0) {
      T *A21 = A + (kb + nb) + kb * lda;
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

// The plain Cholesky (mat_chol, mat_solve_spd, matgb_potrf_dev): float
// orders from 1024 up take their SYRK updates on the tensor cores in the
// FP32-accurate split form (lp 2) unless matgb_plain_tensor_core(0).
int potrf(int64_t n, elem_t *A, int64_t lda, int32_t *info) {
  const int lp = (sizeof(elem_t) == 4 && plain_tc_on() && n >= kPlainTcMinN) ? 2 : -1;
  return potrf_t<elem_t>(n, A, lda, info, lp);
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

int matgb_chol_lookahead(int on) {
  const int prev = g_chol_la;
  if (on >= 0) g_chol_la = on ? 1 : 0;
  return prev;
}

}  // extern "C"
