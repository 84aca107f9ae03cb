// Triangular solve with one right-hand side in a single launch (the
// mat_solve_tril / _tril_unit / _triu / _trilt kernels, mat.h:4580-4803, and
// every refinement step of the mixed-precision solvers).
//
// One CTA per 64-row block of x.  CTAs take blocks in the order they start
// (atomic ticket), so a block only ever waits on blocks owned by CTAs that
// are already running: no deadlock whatever the residency.  A CTA folds in
// the off-diagonal tiles T_bj x_j as their x_j blocks become ready (per-block
// flags, checked for a whole range at a time), then solves its 64x64 diagonal
// block with one warp (x_k broadcast by shuffle, non-unit diagonals divided
// by), publishes x_b and raises its flag.  Flags carry an epoch so they never
// need clearing.  Every wait is bounded: after ~1 s the CTA records an error
// flag and returns.
#include "internal.cuh"

namespace mgb {

constexpr int kTvRows = 64;
constexpr int kTvThreads = 256;
constexpr uint32_t kTvSpinLimit = 1u << 20;  // ~1 s of polling

struct TvState {
  int ticket;
  int err;
  int epoch;
  int pad;
};

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// EL: op(T) lower (forward); TR: op(T) = T^T; UNIT: unit diagonal.
template <typename T, bool EL, bool TR, bool UNIT>
__global__ void __launch_bounds__(kTvThreads)
    trsv_kernel(int64_t n, const T *__restrict__ Tm, int64_t ldt,
                T *__restrict__ x, int *__restrict__ flags,
                TvState *__restrict__ stt, int epoch) {
  __shared__ int sb;
  __shared__ int s_ready;
  __shared__ T part[4][kTvRows];
  __shared__ T Dg[kTvRows][kTvRows + 1];
  __shared__ T xs[kTvRows];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = (int)((n + kTvRows - 1) / kTvRows);
  if (tid == 0) sb = atomicAdd(&stt->ticket, 1);
  __syncthreads();
  const int t = sb;
  if (t >= nb) return;
  const int b = EL ? t : nb - 1 - t;
  const int64_t r0 = (int64_t)b * kTvRows;
  const int rows = (int)((n - r0) < kTvRows ? (n - r0) : kTvRows);
  // op(T)(i, j) in memory
  auto el = [&](int64_t i, int64_t j) -> T {
    return TR ? Tm[j + i * ldt] : Tm[i + j * ldt];
  };

  // partial sums: thread (rr = tid % 64, grp = tid / 64) for !TR, or
  // (cc = tid % 64, grp = tid / 64) for TR
  T acc[kTvRows / 4];
#pragma unroll
  for (int q = 0; q < kTvRows / 4; q++) acc[q] = T(0);
  T accr = T(0);
  int done = 0;  // number of off-diagonal blocks folded in, in solve order
  const int need = t;  // blocks before this one in solve order
  uint32_t spins = 0;
  bool failed = false;
  while (done < need) {
    // how many consecutive blocks (in solve order) are ready from `done`
    if (tid == 0) s_ready = 0x7fffffff;
    __syncthreads();
    {
      const int k = done + tid;
      int ok = 0;
      if (k < need) {
        const int jb = EL ? k : nb - 1 - k;
        ok = ld_acquire(&flags[jb]) == epoch;
      }
      // first not-ready position among the 256 checked
      unsigned bal = __ballot_sync(0xffffffffu, !ok && k < need);
      if (lane == 0) atomicMin(&s_ready, warp * 32 + (bal ? __ffs(bal) - 1 : 32));
    }
    __syncthreads();
    int ready = s_ready;
    if (ready > need - done) ready = need - done;
    if (ready == 0) {
      if (++spins > kTvSpinLimit) {
        failed = true;
        break;
      }
      __nanosleep(100);
      continue;
    }
    for (int q = 0; q < ready; q++) {
      const int k = done + q;
      const int jb = EL ? k : nb - 1 - k;
      const int64_t c0 = (int64_t)jb * kTvRows;
      const int cols = (int)((n - c0) < kTvRows ? (n - c0) : kTvRows);
      if (!TR) {
        // thread: row rr, columns grp*16 .. +16 (coalesced down a column)
        const int rr = tid % kTvRows, grp = tid / kTvRows;
        if (rr < rows) {
#pragma unroll 4
          for (int c = grp * 16; c < grp * 16 + 16; c++)
            if (c < cols) accr = fma(el(r0 + rr, c0 + c), __ldcg(&x[c0 + c]), accr);
        }
      } else {
        // thread: column cc, rows grp*16 .. +16 (coalesced along cc)
        const int cc = tid % kTvRows, grp = tid / kTvRows;
        if (cc < cols) {
          const T xc = __ldcg(&x[c0 + cc]);
#pragma unroll
          for (int q2 = 0; q2 < kTvRows / 4; q2++) {
            const int r = grp * 16 + q2;
            if (r < rows) acc[q2] = fma(el(r0 + r, c0 + cc), xc, acc[q2]);
          }
        }
      }
    }
    done += ready;
  }
  if (failed) {
    if (tid == 0) atomicExch(&stt->err, 1);
    return;
  }
  // reduce partial sums to s[r] for the block's rows
  if (!TR) {
    part[tid / kTvRows][tid % kTvRows] = accr;
  } else {
    // sum over cc: 64 threads (2 warps) per row group; rows grp*16+q2
    const int grp = tid / kTvRows;
#pragma unroll
    for (int q2 = 0; q2 < kTvRows / 4; q2++) {
      T v = acc[q2];
      for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      acc[q2] = v;
    }
    __syncthreads();
    if (lane == 0) {
      const int half = (tid % kTvRows) / 32;  // which warp of the pair
#pragma unroll
      for (int q2 = 0; q2 < kTvRows / 4; q2++) Dg[grp * 16 + q2][half] = acc[q2];
    }
    __syncthreads();
    if (tid < kTvRows) part[0][tid] = Dg[tid][0] + Dg[tid][1];
    if (tid < kTvRows) part[1][tid] = part[2][tid] = part[3][tid] = T(0);
  }
  __syncthreads();
  // diagonal block into shared memory
  for (int e = tid; e < kTvRows * kTvRows; e += kTvThreads) {
    const int i = e % kTvRows, j = e / kTvRows;
    Dg[i][j] = (i < rows && j < rows) ? el(r0 + i, r0 + j) : T(0);
  }
  if (tid < kTvRows)
    xs[tid] = tid < rows ? __ldcg(&x[r0 + tid]) - (part[0][tid] + part[1][tid] +
                                          part[2][tid] + part[3][tid])
                         : T(0);
  __syncthreads();
  if (warp == 0) {
    T y0 = xs[lane], y1 = xs[lane + 32];
    if (EL) {
#pragma unroll 4
      for (int k = 0; k < kTvRows; k++) {
        if (k >= rows) break;
        const int own = k & 31;
        T yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, own);
        if (!UNIT) yk = yk / Dg[k][k];
        if (lane == own) {
          if (k < 32) y0 = yk; else y1 = yk;
        }
        if (lane > k) y0 = fma(-Dg[lane][k], yk, y0);
        if (lane + 32 > k) y1 = fma(-Dg[lane + 32][k], yk, y1);
      }
    } else {
      for (int k = kTvRows - 1; k >= 0; k--) {
        if (k >= rows) continue;
        const int own = k & 31;
        T yk = __shfl_sync(0xffffffffu, k < 32 ? y0 : y1, own);
        if (!UNIT) yk = yk / Dg[k][k];
        if (lane == own) {
          if (k < 32) y0 = yk; else y1 = yk;
        }
        if (lane < k) y0 = fma(-Dg[lane][k], yk, y0);
        if (lane + 32 < k) y1 = fma(-Dg[lane + 32][k], yk, y1);
      }
    }
    if (lane < rows) x[r0 + lane] = y0;
    if (lane + 32 < rows) x[r0 + lane + 32] = y1;
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      st_release(&flags[b], epoch);
    }
  }
}

struct TvBufs {
  int *flags = nullptr;
  TvState *st = nullptr;
  int64_t cap = 0;
  int epoch = 0;
};
static TvBufs g_tv;

template <typename T, bool EL, bool TR, bool UNIT>
static int launch_trsv(int64_t n, const T *Tm, int64_t ldt, T *x) {
  const int nb = (int)((n + kTvRows - 1) / kTvRows);
  if (g_tv.cap < nb) {
    if (g_tv.flags) {
      cudaStreamSynchronize(ctx()->stream);
      cudaFree(g_tv.flags);
    }
    const int64_t cap = nb < 4096 ? 4096 : nb;
    MGB_CUDA(cudaMalloc(&g_tv.flags, cap * sizeof(int) + sizeof(TvState) * 64));
    MGB_CUDA(cudaMemset(g_tv.flags, 0, cap * sizeof(int) + sizeof(TvState) * 64));
    g_tv.st = (TvState *)(g_tv.flags + cap);
    g_tv.cap = cap;
    g_tv.epoch = 0;
  }
  g_tv.epoch++;
  MGB_CUDA(cudaMemsetAsync(&g_tv.st->ticket, 0, sizeof(int), ctx()->stream));
  KtScope kt("trsv", (double)n * n, (double)sizeof(T) * n * n / 2.0);
  trsv_kernel<T, EL, TR, UNIT><<<nb, kTvThreads, 0, ctx()->stream>>>(
      n, Tm, ldt, x, g_tv.flags, g_tv.st, g_tv.epoch);
  MGB_LAUNCHED("trsv");
  return 0;
}

template <typename T>
int trsv_t(bool lower, bool trans, bool unit, int64_t n, const T *Tm,
           int64_t ldt, T *x) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  if (n <= 0) return 0;
  const bool el = lower != trans;
#define MGB_TV(E, R, U)                                                        \
  if (el == E && trans == R && unit == U)                                      \
    return launch_trsv<T, E, R, U>(n, Tm, ldt, x);
  MGB_TV(true, false, false)
  MGB_TV(true, false, true)
  MGB_TV(true, true, false)
  MGB_TV(true, true, true)
  MGB_TV(false, false, false)
  MGB_TV(false, false, true)
  MGB_TV(false, true, false)
  MGB_TV(false, true, true)
#undef MGB_TV
  return MATGB_ERR_ARG;
}

template int trsv_t<float>(bool, bool, bool, int64_t, const float *, int64_t,
                           float *);
template int trsv_t<double>(bool, bool, bool, int64_t, const double *, int64_t,
                            double *);

int trsv_status() {
  if (!g_tv.st) return 0;
  int e = 0;
  MGB_CUDA(cudaMemcpy(&e, &g_tv.st->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    MGB_CUDA(cudaMemset(&g_tv.st->err, 0, sizeof(int)));
    return set_error(MATGB_ERR_TIMEOUT, "triangular solve gave up waiting");
  }
  return 0;
}

}  // namespace mgb
