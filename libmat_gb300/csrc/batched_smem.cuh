// Blocked batched solver with the rows in shared memory: the double build's
// orders 65..128, whose rows do not fit in registers.  The same panel scheme
// as batched_blk.cuh (warp-0 panel with mat_plu's pivot rule, U12 by the
// unit-lower solve, rank-8 updates in step order, back substitution in warp
// 0); thread i owns physical row i of [A | b], kept in shared memory
// (row-major, stride NB + 1 so that a column access is conflict-free), and
// updates it in place.  One system per CTA; at order 128 the system and its
// U take ~220 KB, one CTA per SM.
#pragma once

#include "batched_blk.cuh"

namespace mgb {

template <typename T, int NB>
struct SmemRows {
  BlkSmem<T, NB> b;
  T rows[NB][NB + 1];
};

template <typename T, int NB, int KIND, class Bar = CtaBar>
__device__ int solve_smem(const T *__restrict__ A, int n, const T *__restrict__ b,
                          T *__restrict__ x, SmemRows<T, NB> &S, int i, T eps,
                          Bar bar = Bar()) {
  BlkSmem<T, NB> &sm = S.b;
  T *row = S.rows[i];
  const int warp = i >> 5, lane = i & 31;
  const bool act = i < n;
  // coalesced load: column j of A by all threads
  for (int j = 0; j < n; j++) {
    if (act) {
      T v;
      if (KIND == 1 && j > i)
        v = A[j + (int64_t)i * n];  // upper entry mirrored from the lower
      else
        v = A[i + (int64_t)j * n];
      row[j] = v;
    }
  }
  T rb = act ? b[i] : T(0);
  sm.lr[i] = act ? i : -1;
  if (i == 0) sm.fail = 0;
  for (int K0 = 0; K0 < n; K0 += kBPW) {
    const int live = n - K0;
    const int pw = live < kBPW ? live : kBPW;
    const int tw = live - pw;
    int mylr = sm.lr[i];
    if (mylr >= K0) {
#pragma unroll
      for (int c = 0; c < kBPW; c++) sm.pan[i][c] = c < pw ? row[K0 + c] : T(0);
    }
    bar();
    if (warp == 0) {
      if (!blk_panel<T, NB, KIND>(sm, K0, pw, n, eps) && lane == 0) sm.fail = 1;
    }
    bar();
    if (KIND == 1 && sm.fail) return -1;
    mylr = sm.lr[i];
    if (mylr >= K0 && mylr < K0 + pw) {
      T *rw = sm.raw[mylr - K0];
      for (int j = 0; j < tw; j++) rw[j] = row[K0 + pw + j];
      rw[tw] = rb;
    }
    bar();
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
      const int c = i - (NB - kBPW);
      T *col = sm.ucol + ucoff(K0 + c) + K0;
      for (int c2 = 0; c2 <= c; c2++) col[c2] = sm.pan[sm.pv[c2]][c];
    }
    bar();
    if (mylr >= K0 + pw) {
      T l[kBPW];
      ld8<T>(&sm.pan[i][0], l);
#pragma unroll
      for (int c = 0; c < kBPW; c++) l[c] = c < pw ? l[c] : T(0);
      for (int j = 0; j < tw; j++) {
        T u[kBPW];
        ld8<T>(&sm.u12[j][0], u);
        T v = row[K0 + pw + j];
#pragma unroll
        for (int c = 0; c < kBPW; c++) v = fma(-u[c], l[c], v);
        row[K0 + pw + j] = v;
      }
      T u[kBPW];
      ld8<T>(&sm.u12[tw][0], u);
#pragma unroll
      for (int c = 0; c < kBPW; c++) rb = fma(-u[c], l[c], rb);
    }
  }
  bar();
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

template <typename T, int NB, int KIND>
__global__ void __launch_bounds__(NB, 1)
    batched_smem_kernel(int queue, const int32_t *__restrict__ list,
                        BatchQueues *q, const int32_t *__restrict__ nvec,
                        const int64_t *__restrict__ offA, const T *__restrict__ A,
                        const int64_t *__restrict__ offv, const T *__restrict__ b,
                        T *__restrict__ x, int32_t *__restrict__ status, T eps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemRows<T, NB> &S = *reinterpret_cast<SmemRows<T, NB> *>(smem_raw);
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
    if (n < 1 || n > NB) continue;
    const int st = solve_smem<T, NB, KIND>(A + offA[s], n, b + offv[s], x + offv[s],
                                           S, i, eps);
    if (i == 0) status[s] = st;
    __syncthreads();
  }
}

template <typename T, int NB, int KIND>
int launch_smem_queue(int queue, const int32_t *list, BatchQueues *q,
                      const int32_t *n, const int64_t *offA, const T *A,
                      const int64_t *offv, const T *b, T *x, int32_t *status,
                      T eps) {
  auto k = batched_smem_kernel<T, NB, KIND>;
  const size_t smem = sizeof(SmemRows<T, NB>);
  static bool attr = false;
  if (!attr) {
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    attr = true;
  }
  int per_sm = 0;
  MGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NB, smem));
  if (per_sm < 1) per_sm = 1;
  static const char *names[2][3] = {{"batched_smem_lu_64", "batched_smem_lu_96", "batched_smem_lu_128"},
                                    {"batched_smem_spd_64", "batched_smem_spd_96", "batched_smem_spd_128"}};
  KtScope kt(names[KIND == 1][NB <= 64 ? 0 : NB <= 96 ? 1 : 2], 0.0, 0.0);
  k<<<ctx()->sms * per_sm, NB, smem, ctx()->stream>>>(queue, list, q, n, offA, A,
                                                      offv, b, x, status, eps);
  MGB_LAUNCHED("batched_solve");
  return 0;
}

}  // namespace mgb
