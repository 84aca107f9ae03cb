// Triangular solve with up to 64 right-hand sides in one launch: op(T) X = B
// in place (the refinement's multi-RHS solves with the low-precision factors,
// and mat_solve_tril / _triu / _trilt with several columns, mat.h:4580-4803).
//
// One CTA (256 threads) per 64-row block of X, taken in ticket order as the
// single-RHS solver does (a block only waits on blocks owned by CTAs already
// running, so any residency is deadlock-free).  A CTA stages its diagonal
// block and the reciprocals of its diagonal, then folds in the off-diagonal
// tiles op(T)_bj X_j as their X_j blocks are published: the 64 x 64 matrix
// tile and the 64 x NR block of X_j go to shared memory and every thread
// accumulates a 4 x 4 register tile (two 16-byte shared loads per 16 FMAs).
// The diagonal block is then solved by the eight warps, eight right-hand
// sides each: lane l holds rows l and l + 32, x_k goes out by shuffle and is
// formed with the staged reciprocal (no block barrier inside the solve).
// X_b is written back and the block's flag raised (release); flags carry an
// epoch so they never need clearing, and every wait is bounded (an error
// flag, then the CTA returns).
#include "internal.cuh"

namespace mgb {

constexpr int kTfRB = 64;               // rows per block
constexpr int kTfNR = 64;               // right-hand sides per launch
constexpr uint32_t kTfSpin = 1u << 22;  // ~1 s of polling

struct TfState {
  int ticket;
  int err;
  int pad[2];
};

__device__ __forceinline__ int tf_ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void tf_st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
struct TfSmem {
  T Tt[kTfRB][kTfRB + 1];           // off-diagonal tile, Tt[k][i] = op(T)(i, k)
  __align__(16) T Xs[kTfRB][kTfNR + 4];  // X_j block (row k, rhs c); then S
  T Dg[kTfRB][kTfRB + 1];           // diagonal block, Dg[i][k] = op(T)(i, k)
  T rd[kTfRB];                      // 1 / diagonal
};

// op(T)(i, j) of the column-major T (leading dimension ldt)
template <typename T, bool TR>
__device__ __forceinline__ T tf_at(const T *Tm, int64_t ldt, int64_t i, int64_t j) {
  return TR ? Tm[j + i * ldt] : Tm[i + j * ldt];
}

// Stage the op(T) tile rows [i0, i0+64) x cols [j0, j0+64) as Tt[k][i]
// (zero outside n); coalesced for either orientation.
template <typename T, bool TR>
__device__ __forceinline__ void tf_stage_tile(TfSmem<T> &sm, const T *Tm, int64_t ldt,
                                              int64_t n, int64_t i0, int64_t j0) {
  const int tid = threadIdx.x;
#pragma unroll 4
  for (int e = tid; e < kTfRB * kTfRB; e += 256) {
    // the fast index runs along memory: i for T, k for T^T
    const int f = e & 63, s = e >> 6;
    const int il = TR ? s : f, kl = TR ? f : s;
    const int64_t i = i0 + il, k = j0 + kl;
    sm.Tt[kl][il] = (i < n && k < n) ? tf_at<T, TR>(Tm, ldt, i, k) : T(0);
  }
}

// EL: op(T) lower (forward substitution), else upper (backward); TR: op(T) =
// T^T; UNIT: unit diagonal (not read).  B is n x nr (nr <= 64), in place.
template <typename T, bool EL, bool TR, bool UNIT>
__global__ void __launch_bounds__(256)
    trsm_flag_kernel(int64_t n, int nr, const T *__restrict__ Tm, int64_t ldt,
                     T *__restrict__ B, int64_t ldb, int *__restrict__ flags,
                     TfState *__restrict__ stt, int epoch,
                     const int32_t *__restrict__ info) {
  extern __shared__ __align__(16) unsigned char tf_raw[];
  TfSmem<T> &sm = *reinterpret_cast<TfSmem<T> *>(tf_raw);
  __shared__ int sb, s_fail;
  if (info && *info != 0) return;  // every CTA reads the same flag
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = (int)((n + kTfRB - 1) / kTfRB);
  if (tid == 0) {
    sb = atomicAdd(&stt->ticket, 1);
    s_fail = 0;
  }
  __syncthreads();
  const int b = EL ? sb : nb - 1 - sb;
  const int64_t r0 = (int64_t)b * kTfRB;
  const int rows = (int)((n - r0) < kTfRB ? (n - r0) : kTfRB);
  // diagonal block and reciprocals (independent of X)
#pragma unroll 4
  for (int e = tid; e < kTfRB * kTfRB; e += 256) {
    const int f = e & 63, s = e >> 6;
    const int il = TR ? s : f, kl = TR ? f : s;
    sm.Dg[il][kl] = (il < rows && kl < rows) ? tf_at<T, TR>(Tm, ldt, r0 + il, r0 + kl) : T(0);
  }
  // accumulator: rows 4*ty..+3, right-hand sides 4*tx..+3
  const int ty = tid >> 4, tx = tid & 15;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int64_t r = r0 + 4 * ty + a;
      const int cc = 4 * tx + c;
      acc[a][c] = (r < n && cc < nr) ? B[r + (int64_t)cc * ldb] : T(0);
    }
  __syncthreads();
  if (tid < kTfRB) sm.rd[tid] = (UNIT || tid >= rows) ? T(1) : T(1) / sm.Dg[tid][tid];
  // fold in op(T)_bj X_j for the blocks before b (forward) or after (backward)
  const int need = EL ? b : nb - 1 - b;
  for (int q = 0; q < need; q++) {
    const int jb = EL ? q : nb - 1 - q;
    const int64_t j0 = (int64_t)jb * kTfRB;
    tf_stage_tile<T, TR>(sm, Tm, ldt, n, r0, j0);
    if (tid == 0) {
      uint32_t spins = 0;
      while (tf_ld_acquire(&flags[jb]) != epoch) {
        if (++spins > kTfSpin) {
          s_fail = 1;
          break;
        }
        __nanosleep(32);
      }
    }
    __syncthreads();
    if (s_fail) break;
#pragma unroll 4
    for (int e = tid; e < kTfRB * kTfNR; e += 256) {
      const int kl = e & 63, c = e >> 6;
      const int64_t r = j0 + kl;
      sm.Xs[kl][c] = (r < n && c < nr) ? __ldcg(&B[r + (int64_t)c * ldb]) : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < kTfRB; k++) {
      T tv[4], xv[4];
#pragma unroll
      for (int a = 0; a < 4; a++) tv[a] = sm.Tt[k][4 * ty + a];
#pragma unroll
      for (int c = 0; c < 4; c++) xv[c] = sm.Xs[k][4 * tx + c];
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[a][c] = fma(-tv[a], xv[c], acc[a][c]);
    }
    __syncthreads();
  }
  if (s_fail) {
    if (tid == 0) atomicExch(&stt->err, 1);
    return;
  }
  // the right-hand sides of the block into shared memory, then each warp
  // solves eight of them: lane l holds rows l and l + 32
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) sm.Xs[4 * ty + a][4 * tx + c] = acc[a][c];
  __syncthreads();
  constexpr int CW = kTfNR / 8;  // right-hand sides per warp
  T y0[CW], y1[CW];
#pragma unroll
  for (int c = 0; c < CW; c++) {
    y0[c] = sm.Xs[lane][CW * warp + c];
    y1[c] = sm.Xs[lane + 32][CW * warp + c];
  }
  const int rlo = rows < 32 ? rows : 32;
  if (EL) {
    for (int k = 0; k < rlo; k++) {
      const T rk = sm.rd[k];
      const T d0 = sm.Dg[lane][k], d1 = sm.Dg[lane + 32][k];
#pragma unroll
      for (int c = 0; c < CW; c++) {
        const T xk = __shfl_sync(0xffffffffu, UNIT ? y0[c] : y0[c] * rk, k);
        if (lane == k) y0[c] = xk;
        if (lane > k) y0[c] = fma(-d0, xk, y0[c]);
        y1[c] = fma(-d1, xk, y1[c]);
      }
    }
    for (int k = 32; k < rows; k++) {
      const T rk = sm.rd[k];
      const T d1 = sm.Dg[lane + 32][k];
#pragma unroll
      for (int c = 0; c < CW; c++) {
        const T xk = __shfl_sync(0xffffffffu, UNIT ? y1[c] : y1[c] * rk, k - 32);
        if (lane == k - 32) y1[c] = xk;
        if (lane > k - 32) y1[c] = fma(-d1, xk, y1[c]);
      }
    }
  } else {
    for (int k = rows - 1; k >= 32; k--) {
      const T rk = sm.rd[k];
      const T d0 = sm.Dg[lane][k], d1 = sm.Dg[lane + 32][k];
#pragma unroll
      for (int c = 0; c < CW; c++) {
        const T xk = __shfl_sync(0xffffffffu, UNIT ? y1[c] : y1[c] * rk, k - 32);
        if (lane == k - 32) y1[c] = xk;
        if (lane < k - 32) y1[c] = fma(-d1, xk, y1[c]);
        y0[c] = fma(-d0, xk, y0[c]);
      }
    }
    for (int k = rlo - 1; k >= 0; k--) {
      const T rk = sm.rd[k];
      const T d0 = sm.Dg[lane][k];
#pragma unroll
      for (int c = 0; c < CW; c++) {
        const T xk = __shfl_sync(0xffffffffu, UNIT ? y0[c] : y0[c] * rk, k);
        if (lane == k) y0[c] = xk;
        if (lane < k) y0[c] = fma(-d0, xk, y0[c]);
      }
    }
  }
  // X_b back in place, then the block's flag
#pragma unroll
  for (int c = 0; c < CW; c++) {
    const int cc = CW * warp + c;
    if (cc < nr) {
      if (lane < rows) B[(r0 + lane) + (int64_t)cc * ldb] = y0[c];
      if (lane + 32 < rows) B[(r0 + lane + 32) + (int64_t)cc * ldb] = y1[c];
    }
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) tf_st_release(&flags[b], epoch);
}

struct TfBufs {
  int *flags = nullptr;
  TfState *st = nullptr;
  int64_t cap = 0;
  int epoch = 0;
};
static TfBufs g_tf;

template <typename T, bool EL, bool TR, bool UNIT>
static int launch_tf(int64_t n, int nr, const T *Tm, int64_t ldt, T *B, int64_t ldb,
                     const int32_t *info) {
  const int nb = (int)((n + kTfRB - 1) / kTfRB);
  if (g_tf.cap < nb) {
    if (g_tf.flags) {
      cudaStreamSynchronize(ctx()->stream);
      cudaFree(g_tf.flags);
      g_tf.flags = nullptr;
    }
    const int64_t cap = nb < 4096 ? 4096 : nb;
    MGB_CUDA(cudaMalloc(&g_tf.flags, cap * sizeof(int) + sizeof(TfState) * 4));
    MGB_CUDA(cudaMemset(g_tf.flags, 0, cap * sizeof(int) + sizeof(TfState) * 4));
    g_tf.st = (TfState *)(g_tf.flags + cap);
    g_tf.cap = cap;
    g_tf.epoch = 0;
  }
  g_tf.epoch++;
  auto k = trsm_flag_kernel<T, EL, TR, UNIT>;
  const size_t smem = sizeof(TfSmem<T>);
  MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MGB_CUDA(cudaMemsetAsync(&g_tf.st->ticket, 0, sizeof(int), ctx()->stream));
  KtScope kt("trsm_flag", (double)n * n * nr, (double)sizeof(T) * ((double)n * n / 2.0 + 2.0 * n * nr));
  k<<<nb, 256, smem, ctx()->stream>>>(n, nr, Tm, ldt, B, ldb, g_tf.flags, g_tf.st,
                                      g_tf.epoch, info);
  return launch_check((const void *)k, "trsm_flag", smem);
}

template <typename T>
int trsm_flag_t(bool lower, bool trans, bool unit, int64_t n, int64_t nrhs, const T *Tm,
                int64_t ldt, T *B, int64_t ldb, const int32_t *info) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  if (n <= 0 || nrhs <= 0) return 0;
  const bool el = lower != trans;
  for (int64_t c0 = 0; c0 < nrhs; c0 += kTfNR) {
    const int nr = (int)((nrhs - c0) < kTfNR ? (nrhs - c0) : kTfNR);
    T *Bc = B + c0 * ldb;
#define MGB_TF(E, R, U)                                                        \
  if (el == E && trans == R && unit == U) {                                    \
    MGB_TRY((launch_tf<T, E, R, U>(n, nr, Tm, ldt, Bc, ldb, info)));           \
    continue;                                                                  \
  }
    MGB_TF(true, false, false)
    MGB_TF(true, false, true)
    MGB_TF(true, true, false)
    MGB_TF(true, true, true)
    MGB_TF(false, false, false)
    MGB_TF(false, false, true)
    MGB_TF(false, true, false)
    MGB_TF(false, true, true)
#undef MGB_TF
    return MATGB_ERR_ARG;
  }
  return 0;
}

template int trsm_flag_t<float>(bool, bool, bool, int64_t, int64_t, const float *, int64_t,
                                float *, int64_t, const int32_t *);
template int trsm_flag_t<double>(bool, bool, bool, int64_t, int64_t, const double *, int64_t,
                                 double *, int64_t, const int32_t *);

// Nonzero (and the error recorded) when a multi-RHS solve gave up waiting.
int trsm_flag_status() {
  if (!g_tf.st) return 0;
  int e = 0;
  MGB_CUDA(cudaMemcpy(&e, &g_tf.st->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    MGB_CUDA(cudaMemset(&g_tf.st->err, 0, sizeof(int)));
    return set_error(MATGB_ERR_TIMEOUT, "multi-RHS triangular solve gave up waiting");
  }
  return 0;
}

}  // namespace mgb
