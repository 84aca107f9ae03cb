// Device side of the batched small-system solver (see batched.cu): size
// buckets, per-row register kernels for LU and Cholesky.  Included by one
// translation unit per bucket so the heavily unrolled kernels compile in
// parallel.
#pragma once

#include "internal.cuh"

namespace mgb {

constexpr int kNumBuckets = 5;
constexpr int kNumQueues = 2 * kNumBuckets;  // queue = 2*bucket + kind
__host__ __device__ constexpr int bucket_nb(int b) {
  return b == 0 ? 16 : b == 1 ? 32 : b == 2 ? 64 : b == 3 ? 96 : 128;
}
// Orders above 128 (or below 1) are parked in the 128 bucket's queue but the
// kernels skip them; the driver marks them with status -2.
__host__ __device__ inline int bucket_of(int n) {
  return n <= 16 ? 0 : n <= 32 ? 1 : n <= 64 ? 2 : n <= 96 ? 3 : 4;
}

struct BatchQueues {
  int count[kNumQueues];  // systems per queue
  int next[kNumQueues];   // work counters
  int fill[kNumQueues];   // scatter cursors
};

template <typename T>
__device__ __forceinline__ T bkey(T v, bool first) {
  T a = fabs(v);
  if (a != a) return first ? (T)INFINITY : (T)-1;
  return a;
}

// Threads per system: one per row, at least a full warp (rows >= NB idle).
template <int NB>
struct Tpg {
  static constexpr int v = NB < 32 ? 32 : NB;
};

// Group-wide barrier: the group is one warp for NB <= 32 (several groups per
// CTA), otherwise the whole CTA (one group per CTA).
template <int NB>
__device__ __forceinline__ void gsync() {
  if (NB <= 32) __syncwarp();
  else __syncthreads();
}

template <typename T, int NB>
struct BatchSmem {
  T rowU[2][NB + 1];   // pivot row (incoming row k)
  T rowK[2][NB + 1];   // old row k (goes to row p)
  T wkey[(NB + 31) / 32];
  int widx[(NB + 31) / 32];
  T bc;                // broadcast scalar
  T bc2[2];            // double-buffered broadcast (LU back substitution)
  int flag;
  T Lc[NB * (NB + 1) / 2];  // Cholesky: column k at [k*NB - k(k-1)/2, ...)
};

// The elimination steps are generated by template recursion so that every
// register index is a compile-time constant (a plain loop of 64-128 steps is
// not fully unrolled by the compiler and the row would spill to local memory).
template <typename T, int NB, int K>
struct LuStep {
  // Thread i keeps its physical row; lr is the logical row it currently plays
  // (row exchanges swap roles, not data).  The pivot is the first logical
  // index with max |a| among logical rows >= K (mat__iamax's rule).
  static __device__ __forceinline__ void run(T (&a)[NB], T &rb, int &lr, int n,
                                             int i, bool act,
                                             BatchSmem<T, NB> &sm, T eps) {
    if constexpr (K < NB - 1) {
      if (K >= n - 1) return;  // the reference never searches the last column
      constexpr int buf = K & 1;
      const int lane = i & 31, w = i >> 5;
      const bool cand = act && lr >= K;
      T key = cand ? bkey(a[K], lr == K) : (T)-2;
      int idx = cand ? lr : 0x7fffffff;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const T ok = __shfl_xor_sync(0xffffffffu, key, off);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
        if (ok > key || (ok == key && oi < idx)) { key = ok; idx = oi; }
      }
      int p = idx;
      if constexpr (NB > 32) {
        if (lane == 0) { sm.wkey[w] = key; sm.widx[w] = idx; }
        gsync<NB>();
        T bk = sm.wkey[0];
        p = sm.widx[0];
#pragma unroll
        for (int q = 1; q < NB / 32; q++) {
          const T kq = sm.wkey[q];
          const int iq = sm.widx[q];
          if (kq > bk || (kq == bk && iq < p)) { bk = kq; p = iq; }
        }
      }
      // the pivot row's trailing part is broadcast; roles K and p swap
      const int old = lr;
      if (act && old == p) {
#pragma unroll
        for (int j = K; j < NB; j++) sm.rowU[buf][j] = a[j];
        sm.rowU[buf][NB] = rb;
        lr = K;
      } else if (act && old == K) {
        lr = p;
      }
      gsync<NB>();
      const T piv = sm.rowU[buf][K];
      if (!(fabs(piv) < eps) && act && lr > K) {
        const T l = a[K] * (T(1) / piv);
        a[K] = l;
#pragma unroll
        for (int j = K + 1; j < NB; j++) a[j] = fma(-sm.rowU[buf][j], l, a[j]);
        rb = fma(-sm.rowU[buf][NB], l, rb);
      }
      LuStep<T, NB, K + 1>::run(a, rb, lr, n, i, act, sm, eps);
    }
  }
};

// Back substitution U x = z by logical row, one x_J broadcast per step (J
// descending), the broadcast slot double-buffered so one barrier suffices.
template <typename T, int NB, int J>
struct BackStep {
  static __device__ __forceinline__ void run(const T (&a)[NB], T &rb, T &xi,
                                             int lr, int n, BatchSmem<T, NB> &sm) {
    if constexpr (J >= 0) {
      if (J < n) {
        if (lr == J) {
          xi = rb / a[J];
          sm.bc2[J & 1] = xi;
        }
        gsync<NB>();
        if (lr < J) rb = fma(-a[J], sm.bc2[J & 1], rb);
      }
      BackStep<T, NB, J - 1>::run(a, rb, xi, lr, n, sm);
    }
  }
};

template <typename T, int NB>
__device__ void solve_lu(const T *__restrict__ A, int n, const T *__restrict__ b,
                         T *__restrict__ x, BatchSmem<T, NB> &sm, int i, T eps) {
  const bool act = i < n;
  T a[NB];
  T rb = act ? b[i] : T(0);
#pragma unroll
  for (int j = 0; j < NB; j++) a[j] = (act && j < n) ? A[i + (int64_t)j * n] : T(0);
  int lr = i;
  LuStep<T, NB, 0>::run(a, rb, lr, n, i, act, sm, eps);
  T xi = T(0);
  BackStep<T, NB, NB - 1>::run(a, rb, xi, act ? lr : NB, n, sm);
  if (act) x[lr] = xi;
}

// Cholesky, column K: l_KK = sqrt(a_KK) (status -1 when a_KK <= 0, NaN
// passes as in the reference), column K scaled by 1/l_KK, forward
// substitution fused (y_K = b_K / l_KK), rank-1 update of the lower triangle
// of the owned row with column K broadcast through shared memory.
template <int NB>
__host__ __device__ constexpr int col_off(int k) { return k * NB - k * (k - 1) / 2; }

template <typename T, int NB, int K>
struct CholStep {
  static __device__ __forceinline__ void run(T (&a)[NB], T &rb, int n, int i,
                                             bool act, BatchSmem<T, NB> &sm) {
    if constexpr (K < NB) {
      if (K >= n) return;
      if (i == K) {
        const T d = a[K];
        if (d <= 0) sm.flag = 1;
        const T lkk = sqrt(d);
        a[K] = lkk;
        rb = rb / lkk;
        sm.bc = rb;
        sm.Lc[col_off<NB>(K)] = lkk;
      }
      gsync<NB>();
      if (sm.flag) return;
      const T lkk = sm.Lc[col_off<NB>(K)];
      const T yk = sm.bc;
      if (i > K && act) {
        const T l = a[K] * (T(1) / lkk);
        a[K] = l;
        sm.Lc[col_off<NB>(K) + (i - K)] = l;
        rb = fma(-l, yk, rb);
      }
      gsync<NB>();
      if (i > K && act) {
        const T l = a[K];
#pragma unroll
        for (int j = K + 1; j < NB; j++)
          if (j <= i) a[j] = fma(-l, sm.Lc[col_off<NB>(K) + (j - K)], a[j]);
      }
      CholStep<T, NB, K + 1>::run(a, rb, n, i, act, sm);
    }
  }
};

template <typename T, int NB, int J>
struct CholBackStep {
  static __device__ __forceinline__ void run(T &rb, T &xi, int n, int i,
                                             BatchSmem<T, NB> &sm) {
    if constexpr (J >= 0) {
      if (J < n) {
        if (i == J) {
          xi = rb / sm.Lc[col_off<NB>(J)];
          sm.bc = xi;
        }
        gsync<NB>();
        const T xj = sm.bc;
        // L^T(i, J) = L(J, i) = Lc[col_off(i) + J - i] for i < J
        if (i < J) rb = fma(-sm.Lc[col_off<NB>(i) + (J - i)], xj, rb);
        gsync<NB>();
      }
      CholBackStep<T, NB, J - 1>::run(rb, xi, n, i, sm);
    }
  }
};

template <typename T, int NB>
__device__ void solve_chol(const T *__restrict__ A, int n, const T *__restrict__ b,
                           T *__restrict__ x, BatchSmem<T, NB> &sm, int i,
                           int32_t *status) {
  const bool act = i < n;
  T a[NB];
  T rb = act ? b[i] : T(0);
  // lower triangle of row i (mat_chol reads only the lower triangle)
#pragma unroll
  for (int j = 0; j < NB; j++)
    a[j] = (act && j <= i) ? A[i + (int64_t)j * n] : T(0);
  if (i == 0) sm.flag = 0;
  gsync<NB>();
  CholStep<T, NB, 0>::run(a, rb, n, i, act, sm);
  if (sm.flag) {
    if (i == 0) *status = -1;
    return;
  }
  T xi = T(0);
  CholBackStep<T, NB, NB - 1>::run(rb, xi, n, i, sm);
  if (act) x[i] = xi;
}

// Persistent: every NB-thread group pulls systems of its bucket until the
// queue is empty.  NB <= 32: several independent warp groups per CTA.
template <typename T, int NB, int GROUPS, int KIND>
__global__ void __launch_bounds__(Tpg<NB>::v *GROUPS)
    batched_kernel(int queue, const int32_t *__restrict__ list,
                   BatchQueues *q, const int32_t *__restrict__ nvec,
                   const int64_t *__restrict__ offA, const T *__restrict__ A,
                   const int64_t *__restrict__ offv, const T *__restrict__ b,
                   T *__restrict__ x, int32_t *__restrict__ status, T eps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BatchSmem<T, NB> *smem = reinterpret_cast<BatchSmem<T, NB> *>(smem_raw);
  __shared__ int take[GROUPS];
  constexpr int TPG = Tpg<NB>::v;
  const int g = threadIdx.x / TPG, i = threadIdx.x % TPG;
  int base = 0;
  for (int b2 = 0; b2 < queue; b2++) base += q->count[b2];
  const int cnt = q->count[queue];
  for (;;) {
    if (i == 0) take[g] = atomicAdd(&q->next[queue], 1);
    gsync<NB>();
    const int t = take[g];
    gsync<NB>();
    if (t >= cnt) break;
    const int s = list[base + t];
    const int n = nvec[s];
    if (n < 1 || n > NB) continue;  // unsupported order: reported by the driver
    if (i == 0) status[s] = 0;
    if constexpr (KIND == 1)
      solve_chol<T, NB>(A + offA[s], n, b + offv[s], x + offv[s], smem[g], i,
                        status + s);
    else
      solve_lu<T, NB>(A + offA[s], n, b + offv[s], x + offv[s], smem[g], i, eps);
    gsync<NB>();
  }
}


template <typename T, int NB, int GROUPS, int KIND>
int launch_batched_queue(int queue, const int32_t *list, BatchQueues *q,
                         const int32_t *n, const int64_t *offA, const T *A,
                         const int64_t *offv, const T *b, T *x,
                         int32_t *status, T eps) {
  auto k = batched_kernel<T, NB, GROUPS, KIND>;
  constexpr int threads = Tpg<NB>::v * GROUPS;
  const size_t smem = sizeof(BatchSmem<T, NB>) * GROUPS;
  static bool attr = false;
  if (!attr) {
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    attr = true;
  }
  int per_sm = 0;
  MGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem));
  if (per_sm < 1) per_sm = 1;
  const int grid = ctx()->sms * per_sm;
  static const char *names[2][5] = {
      {"batched_lu_16", "batched_lu_32", "batched_lu_64", "batched_lu_96", "batched_lu_128"},
      {"batched_chol_16", "batched_chol_32", "batched_chol_64", "batched_chol_96", "batched_chol_128"}};
  KtScope kt(names[KIND][NB <= 16 ? 0 : NB <= 32 ? 1 : NB <= 64 ? 2 : NB <= 96 ? 3 : 4], 0.0, 0.0);
  k<<<grid, threads, smem, ctx()->stream>>>(queue, list, q, n, offA, A, offv, b,
                                            x, status, eps);
  MGB_LAUNCHED("batched_solve");
  return 0;
}

// One entry point per (bucket, kind), each in its own translation unit
// batched_nb<NB>_<lu|chol>.cu so the unrolled kernels compile in parallel.
#define MGB_BATCH_DECL(NB, KIND)                                               \
  int batched_bucket_##NB##_##KIND(int queue, const int32_t *list,             \
                                   BatchQueues *q, const int32_t *n,           \
                                   const int64_t *offA, const elem_t *A,       \
                                   const int64_t *offv, const elem_t *b,       \
                                   elem_t *x, int32_t *status);
MGB_BATCH_DECL(16, lu) MGB_BATCH_DECL(16, chol)
MGB_BATCH_DECL(32, lu) MGB_BATCH_DECL(32, chol)
MGB_BATCH_DECL(64, lu) MGB_BATCH_DECL(64, chol)
MGB_BATCH_DECL(96, lu) MGB_BATCH_DECL(96, chol)
MGB_BATCH_DECL(128, lu) MGB_BATCH_DECL(128, chol)
#undef MGB_BATCH_DECL

}  // namespace mgb
