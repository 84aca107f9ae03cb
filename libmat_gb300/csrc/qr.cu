// Householder QR: mat_qr (A = Q R, mat.h:3907-4064) and mat_qr_r (R only,
// mat.h:4066-4192), m >= n, column-major.
//
// Blocked, as the reference's large-matrix path (mat.h:3924-4010): panels of
// kQrNb columns are factored one reflector at a time, H_j = I - tau_j v_j v_j^T
// with the reference's reflector (mat_householder, mat.h:3636-3718: v_j[0] = 1,
// beta = -sign(x0) |x|, tau = -(x0 - beta) / beta, no reflection when
// |x| < MAT_DEFAULT_EPSILON), and the panel's reflectors are gathered into the
// compact WY form H_1 ... H_k = I - Y T Y^T (T upper triangular, built from
// Y^T Y as mat__qr_build_T_ does, mat.h:3772-3830).  The trailing columns of
// R then take one block update R -= Y T^T (Y^T R) and the accumulated Q one
// update Q -= (Q Y) T Y^T (mat.h:3840-3900) -- six products per panel, which
// run on the library's GEMM (the tensor-core split form for large float
// products, the SIMT kernel otherwise).
//
// The panel kernel is one CTA of 512 threads walking the panel's columns;
// for column j it forms |x|^2 (block reduction), the reflector (every thread
// derives beta, v0 and tau from the same reduced value), the dot products of
// v with the panel's remaining columns (per-thread partial sums for up to 32
// columns, one block reduction for all of them) and their rank-1 updates.
// As in the reference, R's entries below the diagonal are what the
// reflections leave there (rounding residue, not set to zero).
#include "internal.cuh"

namespace mgb {

namespace {

constexpr int kQrNb = 32;
constexpr int kQrThreads = 512;  // 128 registers a thread (32 partial sums in double)
constexpr int kQrWarps = kQrThreads / 32;

template <typename T>
__device__ __forceinline__ T block_sum(T v, T *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(~0u, v, off);
  __syncthreads();  // red is free (its last readers are done)
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T s = lane < kQrWarps ? red[lane] : T(0);
  for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(~0u, s, off);
  return s;  // every thread of every warp
}

// Factor the panel R[0:len, 0:kb) (leading dimension ldr) in place; reflector
// j's vector goes to Y[:, j] (len x kb, leading dimension len, zeros above
// row j) and tau[j].
template <typename T>
__global__ void __launch_bounds__(kQrThreads)
    qr_panel_kernel(T *__restrict__ R, int64_t ldr, int64_t len, int kb,
                    T *__restrict__ Y, T *__restrict__ tau, T eps) {
  __shared__ T red[kQrWarps];
  __shared__ T dots[kQrWarps][kQrNb + 1];
  __shared__ T dsum[kQrNb];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int j = 0; j < kb; j++) {
    T *x = R + (int64_t)j * ldr;  // column j
    T *v = Y + (int64_t)j * len;
    // |x|^2 over rows j..len-1
    T ss = 0;
    for (int64_t i = j + tid; i < len; i += kQrThreads) ss += x[i] * x[i];
    const T norm_sq = block_sum(ss, red);
    const T norm_x = sqrt(norm_sq);
    for (int64_t i = tid; i < j; i += kQrThreads) v[i] = T(0);
    if (norm_x < eps) {  // no reflection, v = 0 (a NaN column goes on, as there)
      for (int64_t i = j + tid; i < len; i += kQrThreads) v[i] = T(0);
      if (tid == 0) tau[j] = T(0);
      __syncthreads();
      continue;
    }
    const T x0 = x[j];
    const T beta = x0 >= T(0) ? -norm_x : norm_x;
    const T v0 = x0 - beta;
    const T v0_inv = T(1) / v0;
    const T t = -v0 / beta;
    for (int64_t i = j + tid; i < len; i += kQrThreads)
      v[i] = i == j ? T(1) : x[i] * v0_inv;
    if (tid == 0) tau[j] = t;
    __syncthreads();
    // d_c = v . R[:, c] for the panel's columns c = j..kb-1
    const int nc = kb - j;
    T part[kQrNb];
#pragma unroll
    for (int c = 0; c < kQrNb; c++) part[c] = 0;
    for (int64_t i = j + tid; i < len; i += kQrThreads) {
      const T vi = v[i];
#pragma unroll
      for (int c = 0; c < kQrNb; c++)
        if (c < nc) part[c] = fma(vi, R[i + (int64_t)(j + c) * ldr], part[c]);
    }
#pragma unroll
    for (int c = 0; c < kQrNb; c++) {
      T s = part[c];
      for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(~0u, s, off);
      if (lane == 0) dots[warp][c] = s;
    }
    __syncthreads();
    for (int c = warp; c < nc; c += kQrWarps) {
      T s = lane < kQrWarps ? dots[lane][c] : T(0);
      for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(~0u, s, off);
      if (lane == 0) dsum[c] = t * s;  // w_c = tau * (v . R[:, c])
    }
    __syncthreads();
    // R[:, c] -= w_c v
    for (int64_t i = j + tid; i < len; i += kQrThreads) {
      const T vi = v[i];
      for (int c = 0; c < nc; c++) {
        T *rc = R + (int64_t)(j + c) * ldr + i;
        *rc = fma(-dsum[c], vi, *rc);
      }
    }
    __syncthreads();
  }
}

// T (kb x kb, column-major, upper triangular) of H_1 ... H_kb = I - Y T Y^T
// from G = Y^T Y: T[j][j] = tau_j, T[0:j, j] = -tau_j T[0:j, 0:j] G[0:j, j].
// One warp, lane i owns row i.
template <typename T>
__global__ void qr_build_t_kernel(int kb, const T *__restrict__ G,
                                  const T *__restrict__ tau, T *__restrict__ Tm) {
  __shared__ T t[kQrNb][kQrNb + 1];  // t[i][j]
  const int i = threadIdx.x;
  for (int j = 0; j < kb; j++) {
    T val = 0;
    if (i == j) {
      val = tau[j];
    } else if (i < j) {
      T s = 0;
      for (int l = i; l < j; l++) s = fma(t[i][l], G[l + (int64_t)j * kb], s);
      val = -tau[j] * s;
    }
    if (i < kb) t[i][j] = val;
    __syncwarp();
  }
  for (int j = 0; j < kb; j++)
    if (i < kb) Tm[i + (int64_t)j * kb] = t[i][j];
}

template <typename T>
__global__ void qr_eye_kernel(int64_t m, T *__restrict__ Q, int64_t ldq) {
  const int64_t tot = m * m;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % m, j = e / m;
    Q[i + j * ldq] = i == j ? T(1) : T(0);
  }
}

}  // namespace

// In place on R (m x n, m >= n, holding A on entry); Q (m x m, may be null)
// receives the orthogonal factor.
int qr(int64_t m, int64_t n, elem_t *R, int64_t ldr, elem_t *Q, int64_t ldq) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (m <= 0 || n < 0) return 0;
  cudaStream_t st = cx->stream;
  if (Q) {
    const int64_t b = (m * m + 255) / 256;
    qr_eye_kernel<elem_t><<<(unsigned)(b < (int64_t)cx->sms * 16 ? b : cx->sms * 16),
                            256, 0, st>>>(m, Q, ldq);
    MGB_LAUNCHED("qr_eye");
  }
  if (n == 0) return 0;
  const int64_t nbmax = kQrNb;
  // workspace: Y (m x nb), tau (nb), G and T (nb x nb), W1, W2 (nb x n),
  // C1, C2 (m x nb)
  const size_t cnt = (size_t)m * nbmax + nbmax + 2 * nbmax * nbmax +
                     2 * nbmax * n + 2 * (size_t)m * nbmax;
  elem_t *w = (elem_t *)ws(WS_QR, cnt * sizeof(elem_t));
  if (!w) return MATGB_ERR_NOMEM;
  elem_t *Y = w, *tau = Y + m * nbmax, *G = tau + nbmax, *Tm = G + nbmax * nbmax;
  elem_t *W1 = Tm + nbmax * nbmax, *W2 = W1 + nbmax * n;
  elem_t *C1 = W2 + nbmax * n, *C2 = C1 + m * nbmax;
  for (int64_t jb = 0; jb < n; jb += kQrNb) {
    const int kb = (int)(n - jb < kQrNb ? n - jb : kQrNb);
    const int64_t len = m - jb;
    elem_t *Rp = R + jb + jb * ldr;
    {
      KtScope kt("qr_panel", 4.0 * len * kb * kb, (double)sizeof(elem_t) * 2 * len * kb);
      qr_panel_kernel<elem_t><<<1, kQrThreads, 0, st>>>(Rp, ldr, len, kb, Y, tau,
                                                        kPivotEps);
      MGB_LAUNCHED("qr_panel");
    }
    const int64_t nt = n - jb - kb;  // trailing columns of R
    if (nt <= 0 && !Q) continue;
    // T from G = Y^T Y
    MGB_TRY(gemm(true, false, kb, kb, len, elem_t(1), Y, len, Y, len,
                 elem_t(0), G, kb, 0));
    qr_build_t_kernel<elem_t><<<1, 32, 0, st>>>(kb, G, tau, Tm);
    MGB_LAUNCHED("qr_build_t");
    if (nt > 0) {
      // R[jb:, jb+kb:] -= Y T^T (Y^T R[jb:, jb+kb:])
      elem_t *Rt = R + jb + (jb + kb) * ldr;
      MGB_TRY(gemm(true, false, kb, nt, len, elem_t(1), Y, len, Rt, ldr,
                   elem_t(0), W1, kb, 0));
      MGB_TRY(gemm(true, false, kb, nt, kb, elem_t(1), Tm, kb, W1, kb,
                   elem_t(0), W2, kb, 0));
      MGB_TRY(gemm(false, false, len, nt, kb, elem_t(-1), Y, len, W2, kb,
                   elem_t(1), Rt, ldr, 0));
    }
    if (Q) {
      // Q[:, jb:] -= (Q[:, jb:] Y) T Y^T
      elem_t *Qt = Q + jb * ldq;
      MGB_TRY(gemm(false, false, m, kb, len, elem_t(1), Qt, ldq, Y, len,
                   elem_t(0), C1, m, 0));
      MGB_TRY(gemm(false, false, m, kb, kb, elem_t(1), C1, m, Tm, kb,
                   elem_t(0), C2, m, 0));
      MGB_TRY(gemm(false, true, m, len, kb, elem_t(-1), C2, m, Y, len,
                   elem_t(1), Qt, ldq, 0));
    }
  }
  return 0;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_qr_dev(size_t m, size_t n, mat_elem_t *R, size_t ldr, mat_elem_t *Q,
                 size_t ldq) {
  if (m < n) return set_error(MATGB_ERR_ARG, "qr: requires m >= n");
  if (ldr < m || (Q && ldq < m))
    return set_error(MATGB_ERR_ARG, "qr: leading dimension too small");
  return qr((int64_t)m, (int64_t)n, R, (int64_t)ldr, Q, (int64_t)ldq);
}

}  // extern "C"
