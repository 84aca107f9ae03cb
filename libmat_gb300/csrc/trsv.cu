// Triangular solve with one right-hand side in a single launch (the
// mat_solve_tril / _tril_unit / _triu / _trilt kernels, mat.h:4580-4803, and
// every refinement step of the mixed-precision solvers).
//
// One CTA per RB-row block of x (RB = 64 or 128, 4*RB threads).  CTAs take
// blocks in the order they start (atomic ticket), so a block only ever waits
// on blocks owned by CTAs that are already running: no deadlock whatever the
// residency.  The critical path is the chain of diagonal solves, so
// everything that does not depend on x happens before the wait: the CTA
// stages its diagonal block and the reciprocals of its diagonal in shared
// memory and loads the matrix entries of its next off-diagonal tile into
// registers.  It then folds in the tiles T_bj x_j as their x_j blocks become
// ready (one thread waits on the next flag, all threads then count how many
// more are ready), solves its diagonal block with one warp (x_k broadcast by
// shuffle, multiplication by the staged reciprocal), publishes x_b and raises
// its flag.  Flags carry an epoch so they never need clearing.  Every wait is
// bounded: after ~1 s the CTA records an error flag and returns.
//
// Tile mapping (coalesced either way): op(T) = T, thread (row rr, group g)
// takes columns g*RB/4 .. +RB/4 of row rr; op(T) = T^T (memory contiguous
// along op's columns), warp w takes rows w, w+NW, ... with lanes across
// columns, and the per-row sums are reduced across lanes once at the end.
#include "internal.cuh"

namespace mgb {

constexpr uint32_t kTvSpinLimit = 1u << 22;  // ~1 s of polling

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
// Float solutions are published as 64-bit words (launch epoch << 32 | value
// bits): an aligned 64-bit access is single-copy atomic, so a word that
// carries this launch's epoch carries this launch's value -- no flag and no
// fence between the value and its readiness.
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <typename T, int RB>
struct TvSmem {
  T Dg[RB][RB + 1];  // diagonal block of op(T), row-major
  T rd[RB];          // reciprocals of its diagonal
  T part[4][RB];     // partial sums (op(T) = T)
  T xs[RB];
  T Dinv[RB / 32][32][33];  // INV: inverses of the 32 x 32 diagonal sub-blocks
};

// EL: op(T) lower (forward); TR: op(T) = T^T; UNIT: unit diagonal.
// INV: the diagonal block is solved through the explicit inverses of its
// 32 x 32 sub-blocks, formed while the CTA waits (four short matrix-vector
// products on the critical path instead of RB dependent steps); accuracy then
// depends on those sub-blocks' conditioning, so only the refinement's
// preconditioner uses it.
template <typename T, int RB, bool EL, bool TR, bool UNIT, bool INV>
__global__ void __launch_bounds__(4 * RB)
    trsv_kernel(int64_t n, const T *__restrict__ Tm, int64_t ldt,
                T *__restrict__ x, int *__restrict__ flags,
                TvState *__restrict__ stt, int epoch,
                unsigned long long *__restrict__ xp) {
  // float: x blocks travel as epoch-tagged words in xp (no flags)
  constexpr bool PK = sizeof(T) == 4;
  constexpr int NT = 4 * RB;
  constexpr int NW = NT / 32;
  constexpr int CPT = RB / 4;      // tile entries per thread
  constexpr int RPW = RB / NW;     // TR: rows per warp (8)
  constexpr int LPC = RB / 32;     // TR: columns per lane (2 or 4)
  extern __shared__ __align__(16) unsigned char tv_raw[];
  TvSmem<T, RB> &sm = *reinterpret_cast<TvSmem<T, RB> *>(tv_raw);
  __shared__ int sb, s_fail;
  __shared__ int s_ready[2];  // by iteration parity: reset and read never race
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nb = (int)((n + RB - 1) / RB);
  if (tid == 0) {
    sb = atomicAdd(&stt->ticket, 1);
    s_fail = 0;
  }
  __syncthreads();
  const int t = sb;
  if (t >= nb) return;
  const int b = EL ? t : nb - 1 - t;
  const int64_t r0 = (int64_t)b * RB;
  const int rows = (int)((n - r0) < RB ? (n - r0) : RB);
  auto el = [&](int64_t i, int64_t j) -> T {
    return TR ? Tm[j + i * ldt] : Tm[i + j * ldt];
  };
  // stage the diagonal block (coalesced: contiguous index fastest)
  for (int e = tid; e < RB * RB; e += NT) {
    const int i = TR ? e / RB : e % RB, j = TR ? e % RB : e / RB;
    sm.Dg[i][j] = (i < rows && j < rows) ? el(r0 + i, r0 + j) : T(0);
  }
  __syncthreads();
  if (tid < RB) sm.rd[tid] = (!UNIT && tid < rows) ? T(1) / sm.Dg[tid][tid] : T(1);
  if (INV) {
    __syncthreads();
    // warp s inverts sub-block s: lane j forms column j of its inverse
    if (warp < RB / 32) {
      const int s0 = warp * 32, j = lane;
      T xv[32];
      if (EL) {
#pragma unroll
        for (int i = 0; i < 32; i++) {
          T acc = T(0);
#pragma unroll
          for (int k = 0; k < i; k++) acc = fma(sm.Dg[s0 + i][s0 + k], xv[k], acc);
          const T ri = sm.rd[s0 + i];
          xv[i] = (i == j) ? ri : -ri * acc;
        }
      } else {
#pragma unroll
        for (int i = 31; i >= 0; i--) {
          T acc = T(0);
#pragma unroll
          for (int k = i + 1; k < 32; k++) acc = fma(sm.Dg[s0 + i][s0 + k], xv[k], acc);
          const T ri = sm.rd[s0 + i];
          xv[i] = (i == j) ? ri : -ri * acc;
        }
      }
#pragma unroll
      for (int i = 0; i < 32; i++) sm.Dinv[warp][i][j] = xv[i];
    }
  }

  // this block's right-hand side, read before the wait (only this CTA
  // writes these entries of x)
  const T bv = (tid < rows) ? __ldcg(&x[r0 + tid]) : T(0);
  const int need = t;  // blocks before this one in solve order
  auto tile_col0 = [&](int k) -> int64_t {
    return (int64_t)(EL ? k : nb - 1 - k) * RB;
  };
  // the off-diagonal entries of tile k this thread folds in
  auto load_tile = [&](int k, T (&v)[CPT]) {
    const int64_t c0 = tile_col0(k);
    const int cols = (int)((n - c0) < RB ? (n - c0) : RB);
    if (!TR) {
      const int rr = tid % RB, g = tid / RB;
#pragma unroll
      for (int q = 0; q < CPT; q++) {
        const int c = g * CPT + q;
        v[q] = (rr < rows && c < cols) ? el(r0 + rr, c0 + c) : T(0);
      }
    } else {
#pragma unroll
      for (int a = 0; a < RPW; a++) {
        const int r = warp + a * NW;
#pragma unroll
        for (int m = 0; m < LPC; m++) {
          const int c = lane + 32 * m;
          v[a * LPC + m] = (r < rows && c < cols) ? el(r0 + r, c0 + c) : T(0);
        }
      }
    }
  };
  T cur[CPT], nxt[CPT];
  T acc[TR ? RPW : 1];
#pragma unroll
  for (int a = 0; a < (TR ? RPW : 1); a++) acc[a] = T(0);
  if (need > 0) load_tile(0, cur);

  if constexpr (PK) {
    // every warp folds the tiles in order, polling its own entries of x_k
    // until they carry this launch's epoch (bounded)
    const uint32_t ep = (uint32_t)epoch;
    for (int k = 0; k < need; k++) {
      if (k + 1 < need) load_tile(k + 1, nxt);
      const int64_t c0 = tile_col0(k);
      bool fail = false;
      if (!TR) {
        const int g = tid / RB;
        const int64_t cl = c0 + g * CPT + (lane % CPT);
        const bool in = cl < n;
        unsigned long long v = in ? ld_relaxed_u64(&xp[cl]) : 0ull;
        uint32_t spins = 0;
        while (!__all_sync(0xffffffffu, !in || (uint32_t)(v >> 32) == ep)) {
          if (++spins > kTvSpinLimit) {
            fail = true;
            break;
          }
          if (in && (uint32_t)(v >> 32) != ep) v = ld_relaxed_u64(&xp[cl]);
        }
        if (fail) {
          s_fail = 1;
          break;
        }
        const T xl = in ? (T)__uint_as_float((uint32_t)v) : T(0);
#pragma unroll
        for (int qq = 0; qq < CPT; qq++)
          acc[0] = fma(cur[qq], __shfl_sync(0xffffffffu, xl, qq), acc[0]);
      } else {
        unsigned long long v[LPC];
        bool in[LPC];
#pragma unroll
        for (int m = 0; m < LPC; m++) {
          const int64_t c = c0 + lane + 32 * m;
          in[m] = c < n;
          v[m] = in[m] ? ld_relaxed_u64(&xp[c]) : 0ull;
        }
        uint32_t spins = 0;
        for (;;) {
          bool ok = true;
#pragma unroll
          for (int m = 0; m < LPC; m++) ok = ok && (!in[m] || (uint32_t)(v[m] >> 32) == ep);
          if (__all_sync(0xffffffffu, ok)) break;
          if (++spins > kTvSpinLimit) {
            fail = true;
            break;
          }
#pragma unroll
          for (int m = 0; m < LPC; m++)
            if (in[m] && (uint32_t)(v[m] >> 32) != ep) v[m] = ld_relaxed_u64(&xp[c0 + lane + 32 * m]);
        }
        if (fail) {
          s_fail = 1;
          break;
        }
        T xv[LPC];
#pragma unroll
        for (int m = 0; m < LPC; m++) xv[m] = in[m] ? (T)__uint_as_float((uint32_t)v[m]) : T(0);
#pragma unroll
        for (int a = 0; a < RPW; a++)
#pragma unroll
          for (int m = 0; m < LPC; m++) acc[a] = fma(cur[a * LPC + m], xv[m], acc[a]);
      }
#pragma unroll
      for (int qq = 0; qq < CPT; qq++) cur[qq] = nxt[qq];
    }
    __syncthreads();
  }
  int done = PK ? need : 0, par = 0;
  while (done < need) {
    // wait for tile `done`, then count the ready tiles after it
    if (tid == 0) {
      const int jb = EL ? done : nb - 1 - done;
      uint32_t spins = 0;
      while (ld_acquire(&flags[jb]) != epoch) {
        if (++spins > kTvSpinLimit) {
          s_fail = 1;
          break;
        }
        __nanosleep(32);
      }
      s_ready[par] = 0x7fffffff;
    }
    __syncthreads();
    if (s_fail) break;
    if (need - done > 1) {  // more than one tile pending: count the ready ones
      const int k = done + 1 + tid;
      int ok = 0;
      if (k < need) ok = ld_acquire(&flags[EL ? k : nb - 1 - k]) == epoch;
      const unsigned bal = __ballot_sync(0xffffffffu, !ok && k < need);
      if (lane == 0 && (bal || warp == NW - 1))
        atomicMin(&s_ready[par], warp * 32 + (bal ? __ffs(bal) - 1 : 32));
      __syncthreads();
    }
    int ready = need - done > 1 ? 1 + s_ready[par] : 1;
    par ^= 1;
    if (ready > need - done) ready = need - done;
    for (int q = 0; q < ready; q++) {
      const int k = done + q;
      if (k + 1 < need) load_tile(k + 1, nxt);
      const int64_t c0 = tile_col0(k);
      if (!TR) {
        // the warp's CPT entries of x_k: one coalesced load, then shuffles
        // (a warp's threads share g)
        const int g = tid / RB;
        const int64_t cl = c0 + g * CPT + (lane % CPT);
        const T xl = cl < n ? __ldcg(&x[cl]) : T(0);
#pragma unroll
        for (int qq = 0; qq < CPT; qq++)
          acc[0] = fma(cur[qq], __shfl_sync(0xffffffffu, xl, qq), acc[0]);
      } else {
        T xv[LPC];
#pragma unroll
        for (int m = 0; m < LPC; m++) {
          const int64_t c = c0 + lane + 32 * m;
          xv[m] = c < n ? __ldcg(&x[c]) : T(0);
        }
#pragma unroll
        for (int a = 0; a < RPW; a++)
#pragma unroll
          for (int m = 0; m < LPC; m++) acc[a] = fma(cur[a * LPC + m], xv[m], acc[a]);
      }
#pragma unroll
      for (int qq = 0; qq < CPT; qq++) cur[qq] = nxt[qq];
    }
    done += ready;
  }
  if (s_fail) {
    if (tid == 0) atomicExch(&stt->err, 1);
    return;
  }
  // s = b - (sum of the folded tiles) for the block's rows
  if (!TR) {
    sm.part[tid / RB][tid % RB] = acc[0];
  } else {
#pragma unroll
    for (int a = 0; a < RPW; a++) {
      T v = acc[a];
      for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0) sm.part[0][warp + a * NW] = v;
    }
  }
  __syncthreads();
  if (tid < RB) {
    T s = T(0);
    if (tid < rows) {
      s = sm.part[0][tid];
      if (!TR) s += sm.part[1][tid] + sm.part[2][tid] + sm.part[3][tid];
      s = bv - s;
    }
    sm.xs[tid] = s;
  }
  __syncthreads();
  if (warp == 0) {
    constexpr int YR = RB / 32;  // rows per lane
    T y[YR];
#pragma unroll
    for (int m = 0; m < YR; m++) y[m] = sm.xs[lane + 32 * m];
    if (INV) {
      // sub-block by sub-block: y_s = Dinv_s t_s, then fold y_s into the
      // sub-blocks still to come
#pragma unroll
      for (int q = 0; q < YR; q++) {
        const int sb = EL ? q : YR - 1 - q;
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < 32; k++)
          acc = fma(sm.Dinv[sb][lane][k], __shfl_sync(0xffffffffu, y[sb], k), acc);
        y[sb] = acc;
#pragma unroll
        for (int k = 0; k < 32; k++) {
          const T yk = __shfl_sync(0xffffffffu, y[sb], k);
#pragma unroll
          for (int m = 0; m < YR; m++)
            if (EL ? m > sb : m < sb)
              y[m] = fma(-sm.Dg[lane + 32 * m][sb * 32 + k], yk, y[m]);
        }
      }
    } else if (EL) {
#pragma unroll
      for (int m0 = 0; m0 < YR; m0++) {
#pragma unroll 8
        for (int kk = 0; kk < 32; kk++) {
          const int k = m0 * 32 + kk;
          if (k < rows) {
            T yk = __shfl_sync(0xffffffffu, y[m0], kk);
            if (!UNIT) yk *= sm.rd[k];
            if (lane == kk) y[m0] = yk;
#pragma unroll
            for (int m = 0; m < YR; m++)
              if (lane + 32 * m > k) y[m] = fma(-sm.Dg[lane + 32 * m][k], yk, y[m]);
          }
        }
      }
    } else {
#pragma unroll
      for (int m0 = YR - 1; m0 >= 0; m0--) {
#pragma unroll 8
        for (int kk = 31; kk >= 0; kk--) {
          const int k = m0 * 32 + kk;
          if (k < rows) {
            T yk = __shfl_sync(0xffffffffu, y[m0], kk);
            if (!UNIT) yk *= sm.rd[k];
            if (lane == kk) y[m0] = yk;
#pragma unroll
            for (int m = 0; m < YR; m++)
              if (lane + 32 * m < k) y[m] = fma(-sm.Dg[lane + 32 * m][k], yk, y[m]);
          }
        }
      }
    }
#pragma unroll
    for (int m = 0; m < YR; m++)
      if (lane + 32 * m < rows) x[r0 + lane + 32 * m] = y[m];
    if constexpr (PK) {
#pragma unroll
      for (int m = 0; m < YR; m++)
        if (lane + 32 * m < rows)
          st_relaxed_u64(&xp[r0 + lane + 32 * m],
                         ((unsigned long long)(uint32_t)epoch << 32) |
                             __float_as_uint((float)y[m]));
    } else {
      __syncwarp();
      if (lane == 0) {
        __threadfence();
        st_release(&flags[b], epoch);
      }
    }
  }
}

struct TvBufs {
  int *flags = nullptr;
  TvState *st = nullptr;
  int64_t cap = 0;
  int epoch = 0;
  unsigned long long *xp = nullptr;  // epoch-tagged float solutions
  int64_t xcap = 0;
};
static TvBufs g_tv;

template <typename T, int RB, bool EL, bool TR, bool UNIT, bool INV>
static int launch_trsv(int64_t n, const T *Tm, int64_t ldt, T *x) {
  const int nb = (int)((n + RB - 1) / RB);
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
  unsigned long long *xp = nullptr;
  if constexpr (sizeof(T) == 4) {
    const int64_t need = (int64_t)nb * RB;
    if (g_tv.xcap < need) {
      if (g_tv.xp) {
        cudaStreamSynchronize(ctx()->stream);
        cudaFree(g_tv.xp);
        g_tv.xp = nullptr;
        g_tv.xcap = 0;
      }
      const int64_t cap = need < 65536 ? 65536 : need;
      MGB_CUDA(cudaMalloc(&g_tv.xp, cap * sizeof(unsigned long long)));
      // epoch 0 is never a launch's epoch
      MGB_CUDA(cudaMemset(g_tv.xp, 0, cap * sizeof(unsigned long long)));
      g_tv.xcap = cap;
    }
    xp = g_tv.xp;
  }
  g_tv.epoch++;
  auto k = trsv_kernel<T, RB, EL, TR, UNIT, INV>;
  const size_t smem = sizeof(TvSmem<T, RB>);
  MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
  MGB_CUDA(cudaMemsetAsync(&g_tv.st->ticket, 0, sizeof(int), ctx()->stream));
  KtScope kt(INV ? "trsv_inv" : "trsv", (double)n * n, (double)sizeof(T) * n * n / 2.0);
  k<<<nb, 4 * RB, smem, ctx()->stream>>>(n, Tm, ldt, x, g_tv.flags, g_tv.st,
                                         g_tv.epoch, xp);
  return launch_check((const void *)k, "trsv", smem);
}

// Block rows: 128 once the chain of diagonal solves (n / RB steps) is long.
static int g_tv_rb_override = 0;

template <typename T>
int trsv_t(bool lower, bool trans, bool unit, int64_t n, const T *Tm,
           int64_t ldt, T *x, bool inv) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  if (n <= 0) return 0;
  const bool el = lower != trans;
  // 128-row blocks (512 threads) only in float: the double tiles would not
  // fit the 128 registers a thread may then use
  int rb = g_tv_rb_override ? g_tv_rb_override : (n >= 4096 ? 128 : 64);
  if (sizeof(T) != 4) rb = 64;
#define MGB_TV(E, R, U)                                                        \
  if (el == E && trans == R && unit == U) {                                    \
    if constexpr (sizeof(T) == 4) {                                            \
      if (inv)                                                                 \
        return rb == 128 ? launch_trsv<T, 128, E, R, U, true>(n, Tm, ldt, x)   \
                         : launch_trsv<T, 64, E, R, U, true>(n, Tm, ldt, x);   \
      if (rb == 128) return launch_trsv<T, 128, E, R, U, false>(n, Tm, ldt, x); \
    }                                                                          \
    return launch_trsv<T, 64, E, R, U, false>(n, Tm, ldt, x);                  \
  }
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
                           float *, bool);
template int trsv_t<double>(bool, bool, bool, int64_t, const double *, int64_t,
                            double *, bool);

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

// Block-row size of the single-launch triangular solve (64 or 128; 0 picks
// by size).  For measurement.
extern "C" int matgb_trsv_block_rows(int rb) {
  if (rb != 0 && rb != 64 && rb != 128) return MATGB_ERR_ARG;
  mgb::g_tv_rb_override = rb;
  return 0;
}
