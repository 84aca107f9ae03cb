// Blocked form of the batched small-system solver for orders 33..128 (see
// batched.cu): one system per CTA of NB threads, thread i owning physical row
// i of [A | b] in registers (a shifted frame: before the panel at column K0
// the row holds columns K0.. in a[0..], so every register index is static).
//
// Right-looking LU in panels of kBPW = 8 columns -- the reference's own
// scheme (mat__plu_blocked_, mat.h:4201-4289: panel factorisation with
// partial pivoting, U12 by a unit-lower solve with L11, then the rank-8
// update of the trailing rows), with the right-hand side carried as one more
// trailing column so the forward substitution happens on the way:
//   1. every live row stages its 8 panel entries in shared memory; barrier;
//   2. warp 0 factors the panel alone, 2-4 rows a lane, with warp shuffles
//      only: per column the pivot (mat_plu's rule: first logical row of the
//      largest |a| among rows K.., NaN at the top wins, NaN below never, the
//      last column not searched) by two redux operations on order-preserving
//      keys, the pivot row by shuffles, rows trading roles (logical row
//      numbers) instead of data, multipliers a * (1 / pivot); a pivot below
//      MAT_DEFAULT_EPSILON is swapped in but its column is neither scaled
//      nor applied inside the panel, and its raw entries still act as L in
//      the trailing update, exactly as mat__plu_blocked_ does; barrier;
//   3. the panel's 8 pivot rows stage their trailing entries; barrier;
//   4. thread j solves trailing column j of L11 U12 = A12 (the rank-1 steps
//      in the unblocked order, so the arithmetic is that of the unblocked
//      elimination) and files U12 by columns for the back substitution;
//      barrier;
//   5. every row below the panel takes its rank-8 update, the eight FMAs of
//      an entry in step order (U12 read by broadcast from shared memory).
// Four barriers per 8 columns (the Gauss-Jordan form this replaces took one
// per column and did half again the FMAs).  Warp 0 then back-substitutes
// U x = y column by column with shuffles.
//
// SPD systems (KIND 1): the symmetric matrix rebuilt from the lower triangle
// (what mat_chol reads), no row exchanges; a pivot -- the Schur-complement
// diagonal mat_chol tests -- <= 0 gives status -1 with x untouched (NaN
// passes, as there).
#pragma once

#include "batched_kernels.cuh"

namespace mgb {

constexpr int kBPW = 8;

template <typename T, int NB>
struct BlkSmem {
  __align__(16) T pan[NB][kBPW];     // panel entries by physical row
  __align__(16) T raw[kBPW][NB + 4]; // pivot rows' trailing entries, rhs last
  __align__(16) T u12[NB + 4][kBPW]; // U12 by trailing column (rhs last)
  T ucol[NB * (NB + 1) / 2];         // U by columns: U[i][j] at j(j+1)/2 + i
  T yv[NB];                          // forward-eliminated rhs, by logical row
  T xv[NB];
  int lr[NB];                        // logical row of each physical row
  int pv[kBPW];                      // physical row of logical row K0 + c
  int fail;                          // SPD: a pivot <= 0 was met
};

__device__ __forceinline__ int ucoff(int j) { return j * (j + 1) / 2; }

// The barrier of the threads solving one system: the whole CTA, or a named
// barrier over one group of NB threads (several systems per CTA).
struct CtaBar {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct GroupBar {
  int id, count;  // named barrier id (1..15) and its thread count
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  }
};

// 8 consecutive values to / from 16-byte aligned shared memory, register
// arrays indexed statically only (no address of a register array is taken)
template <typename T>
__device__ __forceinline__ void st8(T *dst, T v0, T v1, T v2, T v3, T v4, T v5,
                                    T v6, T v7) {
  if constexpr (sizeof(T) == 4) {
    reinterpret_cast<float4 *>(dst)[0] = make_float4(v0, v1, v2, v3);
    reinterpret_cast<float4 *>(dst)[1] = make_float4(v4, v5, v6, v7);
  } else {
    reinterpret_cast<double2 *>(dst)[0] = make_double2(v0, v1);
    reinterpret_cast<double2 *>(dst)[1] = make_double2(v2, v3);
    reinterpret_cast<double2 *>(dst)[2] = make_double2(v4, v5);
    reinterpret_cast<double2 *>(dst)[3] = make_double2(v6, v7);
  }
}
template <typename T>
__device__ __forceinline__ void ld8(const T *src, T (&o)[kBPW]) {
  if constexpr (sizeof(T) == 4) {
    const float4 a = reinterpret_cast<const float4 *>(src)[0];
    const float4 b = reinterpret_cast<const float4 *>(src)[1];
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
    o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
  } else {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const double2 a = reinterpret_cast<const double2 *>(src)[k];
      o[2 * k] = a.x;
      o[2 * k + 1] = a.y;
    }
  }
}

// Warp 0: factor the panel [K0, K0 + pw) of rows with logical index >= K0.
// Returns false (SPD only) when a pivot <= 0 was met.
template <typename T, int NB, int KIND>
__device__ __forceinline__ bool blk_panel(BlkSmem<T, NB> &sm, int K0, int pw,
                                          int n, T eps) {
  constexpr int RPL = NB / 32;
  const int lane = threadIdx.x & 31;
  T p[RPL][kBPW];
  int plr[RPL];
#pragma unroll
  for (int q = 0; q < RPL; q++) {
    const int r = lane + 32 * q;
    plr[q] = sm.lr[r];
#pragma unroll
    for (int c = 0; c < kBPW; c++) p[q][c] = plr[q] >= K0 ? sm.pan[r][c] : T(0);
  }
  bool ok = true;
#pragma unroll
  for (int c = 0; c < kBPW; c++) {
    if (c >= pw) break;
    const int K = K0 + c;
    int piv_lr = K;
    if (KIND == 0 && K < n - 1) {
      if constexpr (sizeof(T) == 4) {
        unsigned bk = 0u;
        int bl = 0x7fffffff;
#pragma unroll
        for (int q = 0; q < RPL; q++) {
          const bool cand = plr[q] >= K;
          const unsigned key = cand ? fkey((float)p[q][c], plr[q] == K) : 0u;
          if (key > bk || (key == bk && key != 0u && plr[q] < bl)) {
            bk = key;
            bl = plr[q];
          }
        }
        const unsigned wk = __reduce_max_sync(0xffffffffu, bk);
        piv_lr = (int)__reduce_min_sync(
            0xffffffffu, (bk == wk && wk != 0u) ? (unsigned)bl : 0x7fffffffu);
      } else {
        T bk = T(-2);
        int bl = 0x7fffffff;
#pragma unroll
        for (int q = 0; q < RPL; q++) {
          if (plr[q] >= K) {
            const T key = bkey(p[q][c], plr[q] == K);
            if (key > bk || (key == bk && plr[q] < bl)) {
              bk = key;
              bl = plr[q];
            }
          }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const T ok2 = __shfl_xor_sync(0xffffffffu, bk, off);
          const int oi = __shfl_xor_sync(0xffffffffu, bl, off);
          if (ok2 > bk || (ok2 == bk && oi < bl)) {
            bk = ok2;
            bl = oi;
          }
        }
        piv_lr = bl;
      }
    }
    // the lane (and slot) holding the pivot row
    int qs = -1;
#pragma unroll
    for (int q = 0; q < RPL; q++)
      if (plr[q] == piv_lr) qs = q;
    const unsigned bal = __ballot_sync(0xffffffffu, qs >= 0);
    const int src = __ffs(bal) - 1;
    T prow[kBPW];
#pragma unroll
    for (int cc = 0; cc < kBPW; cc++) {
      T v = T(0);
#pragma unroll
      for (int q = 0; q < RPL; q++)
        if (q == qs) v = p[q][cc];
      prow[cc] = __shfl_sync(0xffffffffu, v, src);
    }
    const int pq = __shfl_sync(0xffffffffu, qs, src);
    if (lane == 0) sm.pv[c] = src + 32 * pq;
    // roles: the pivot row becomes logical row K, the row that was K takes
    // the pivot's old place
#pragma unroll
    for (int q = 0; q < RPL; q++) {
      if (plr[q] == piv_lr)
        plr[q] = K;
      else if (plr[q] == K)
        plr[q] = piv_lr;
    }
    const T piv = prow[c];
    if (KIND == 1 && piv <= T(0)) {  // NaN passes, as in mat_chol
      ok = false;
      break;
    }
    const bool elim = KIND == 1 || !(fabs(piv) < eps);
    const T inv = T(1) / piv;
#pragma unroll
    for (int q = 0; q < RPL; q++) {
      if (plr[q] > K && elim) {
        const T l = p[q][c] * inv;
        p[q][c] = l;
#pragma unroll
        for (int cc = c + 1; cc < kBPW; cc++) p[q][cc] = fma(-prow[cc], l, p[q][cc]);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < RPL; q++) {
    const int r = lane + 32 * q;
    if (sm.lr[r] >= K0) {
#pragma unroll
      for (int c = 0; c < kBPW; c++) sm.pan[r][c] = p[q][c];
    }
    sm.lr[r] = plr[q];
  }
  return ok;
}

// Solve one system of order n (NB - 31 <= n <= NB in practice; any n <= NB
// works) with the CTA's NB threads; returns the status (0, or -1: SPD
// system not positive definite, x untouched).
template <typename T, int NB, int KIND, class Bar = CtaBar>
__device__ int solve_blk(const T *__restrict__ A, int n, const T *__restrict__ b,
                         T *__restrict__ x, BlkSmem<T, NB> &sm, int i, T eps,
                         Bar bar = Bar()) {
  constexpr int W = VecOf<T>::w;
  const int warp = i >> 5, lane = i & 31;
  const bool act = i < n;
  T a[NB];
  T rb = act ? b[i] : T(0);
#pragma unroll
  for (int j = 0; j < NB; j++) {
    T v = T(0);
    if (act && j < n) {
      if (KIND == 1 && j > i)
        v = A[j + (int64_t)i * n];  // upper entry mirrored from the lower
      else
        v = A[i + (int64_t)j * n];
    }
    a[j] = v;
  }
  sm.lr[i] = act ? i : -1;
  if (i == 0) sm.fail = 0;
  // (the barrier of phase 1 orders these writes before the panel reads them)
  for (int K0 = 0; K0 < n; K0 += kBPW) {
    const int live = n - K0;
    const int pw = live < kBPW ? live : kBPW;
    const int tw = live - pw;  // trailing columns (0 on the last panel)
    // 1. stage the panel entries of every live row
    int mylr = sm.lr[i];
    if (mylr >= K0) st8<T>(&sm.pan[i][0], a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7]);
    bar();
    // 2. the panel, in warp 0
    if (warp == 0) {
      if (!blk_panel<T, NB, KIND>(sm, K0, pw, n, eps) && lane == 0) sm.fail = 1;
    }
    bar();
    if (KIND == 1 && sm.fail) return -1;
    mylr = sm.lr[i];
    // 3. the panel's pivot rows stage their trailing entries and rhs
    if (mylr >= K0 && mylr < K0 + pw) {
      T *rw = sm.raw[mylr - K0];
      if (tw > 0) {  // then pw == 8: trailing column j is a[8 + j]
#pragma unroll
        for (int j0 = 0; j0 + kBPW < NB; j0 += W) {
          if (j0 < tw) {
            T v[W];
#pragma unroll
            for (int q = 0; q < W; q++)
              v[q] = j0 + q + kBPW < NB ? a[j0 + q + kBPW] : T(0);
            VecOf<T>::put(rw + j0, v);
          }
        }
      }
      rw[tw] = rb;  // after the vector stores (one may run past tw)
    }
    bar();
    // 4. U12 column by column (thread j), rhs last; U filed by columns
    if (i <= tw) {
      T u[kBPW];
#pragma unroll
      for (int c = 0; c < kBPW; c++) {
        T v = T(0);
        if (c < pw) {
          v = sm.raw[c][i];
          const int pr = sm.pv[c];
#pragma unroll
          for (int c2 = 0; c2 < c; c2++) v = fma(-sm.pan[pr][c2], u[c2], v);
        }
        u[c] = v;
      }
      st8<T>(&sm.u12[i][0], u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7]);
      if (i < tw) {
        T *col = sm.ucol + ucoff(K0 + pw + i) + K0;
#pragma unroll
        for (int c = 0; c < kBPW; c++)
          if (c < pw) col[c] = u[c];
      } else {
#pragma unroll
        for (int c = 0; c < kBPW; c++)
          if (c < pw) sm.yv[K0 + c] = u[c];
      }
    }
    if (i >= NB - kBPW && i - (NB - kBPW) < pw) {
      // U11's column c (threads NB-8.. are otherwise idle here)
      const int c = i - (NB - kBPW);
      T *col = sm.ucol + ucoff(K0 + c) + K0;
      for (int c2 = 0; c2 <= c; c2++) col[c2] = sm.pan[sm.pv[c2]][c];
    }
    bar();
    // 5. rank-8 update of the rows below the panel, then the frame shifts
    if (mylr >= K0 + pw) {
      T l[kBPW];
      ld8<T>(&sm.pan[i][0], l);
#pragma unroll
      for (int c = 0; c < kBPW; c++) l[c] = c < pw ? l[c] : T(0);
      if (tw > 0) {
#pragma unroll
        for (int j0 = 0; j0 + kBPW < NB; j0 += 4) {
          if (j0 < tw) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const int j = j0 + q;
              if (j + kBPW < NB) {
                T u[kBPW];
                ld8<T>(&sm.u12[j][0], u);
                T v = a[j + kBPW];
#pragma unroll
                for (int c = 0; c < kBPW; c++) v = fma(-u[c], l[c], v);
                a[j] = v;
              }
            }
          }
        }
      }
      T u[kBPW];
      ld8<T>(&sm.u12[tw][0], u);
#pragma unroll
      for (int c = 0; c < kBPW; c++) rb = fma(-u[c], l[c], rb);
    }
  }
  bar();
  // back substitution U x = y in warp 0: column by column, lane l holding
  // the partial sums of rows l, l + 32, ...
  if (warp == 0) {
    constexpr int RPL = NB / 32;
    T s[RPL];
#pragma unroll
    for (int q = 0; q < RPL; q++) {
      const int r = lane + 32 * q;
      s[q] = r < n ? sm.yv[r] : T(0);
    }
    for (int j = n - 1; j >= 0; j--) {
      const int qo = j >> 5;
      T v = T(0);
#pragma unroll
      for (int q = 0; q < RPL; q++)
        if (q == qo) v = s[q];
      const T xj = __shfl_sync(0xffffffffu, v, j & 31) / sm.ucol[ucoff(j) + j];
      if (lane == 0) sm.xv[j] = xj;
      const T *col = sm.ucol + ucoff(j);
#pragma unroll
      for (int q = 0; q < RPL; q++) {
        const int r = lane + 32 * q;
        if (r < j) s[q] = fma(-col[r], xj, s[q]);
      }
    }
  }
  bar();
  if (act) x[i] = sm.xv[i];
  return 0;
}

// Persistent: each CTA (one system at a time) pulls systems of its queue.
template <typename T, int NB, int KIND, int MINB>
__global__ void __launch_bounds__(NB, MINB)
    batched_blk_kernel(int queue, const int32_t *__restrict__ list,
                       BatchQueues *q, const int32_t *__restrict__ nvec,
                       const int64_t *__restrict__ offA, const T *__restrict__ A,
                       const int64_t *__restrict__ offv, const T *__restrict__ b,
                       T *__restrict__ x, int32_t *__restrict__ status, T eps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BlkSmem<T, NB> &sm = *reinterpret_cast<BlkSmem<T, NB> *>(smem_raw);
  __shared__ int take;
  const int i = threadIdx.x;
  int base = 0;
  for (int b2 = 0; b2 < queue; b2++) base += q->count[b2];
  const int cnt = q->count[queue];
  for (;;) {
    if (i == 0) take = atomicAdd(&q->next[queue], 1);
    __syncthreads();
    const int t = take;
    __syncthreads();
    if (t >= cnt) break;
    const int s = list[base + t];
    const int n = nvec[s];
    if (n < 1 || n > NB) continue;  // unsupported order: reported by the driver
    const int st = solve_blk<T, NB, KIND>(A + offA[s], n, b + offv[s], x + offv[s],
                                          sm, i, eps);
    if (i == 0) status[s] = st;
    __syncthreads();  // shared memory is reused by the next system
  }
}

template <typename T, int NB, int KIND, int MINB>
int launch_blk_queue(int queue, const int32_t *list, BatchQueues *q,
                     const int32_t *n, const int64_t *offA, const T *A,
                     const int64_t *offv, const T *b, T *x, int32_t *status,
                     T eps, int ctas_per_sm = 0) {
  auto k = batched_blk_kernel<T, NB, KIND, MINB>;
  const size_t smem = sizeof(BlkSmem<T, NB>);
  static bool attr = false;
  if (!attr) {
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    attr = true;
  }
  int per_sm = 0;
  MGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NB, smem));
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  if (per_sm < 1) per_sm = 1;
  const int grid = ctx()->sms * per_sm;
  static const char *names[2][3] = {{"batched_blk_lu_64", "batched_blk_lu_96", "batched_blk_lu_128"},
                                    {"batched_blk_spd_64", "batched_blk_spd_96", "batched_blk_spd_128"}};
  KtScope kt(names[KIND == 1][NB <= 64 ? 0 : NB <= 96 ? 1 : 2], 0.0, 0.0);
  k<<<grid, NB, smem, ctx()->stream>>>(queue, list, q, n, offA, A, offv, b, x,
                                       status, eps);
  MGB_LAUNCHED("batched_solve");
  return 0;
}

}  // namespace mgb
