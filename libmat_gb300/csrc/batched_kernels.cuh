// Device side of the batched small-system solver (see batched.cu): size
// buckets and the per-row register kernel shared by the general (partial
// pivoting) and SPD systems.  Included by one translation unit per bucket so
// the kernels compile in parallel.
#pragma once

#include <type_traits>

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
  // mixed-precision (tensor-core) kernels: refinement corrections taken,
  // systems left above the FP32-level residual, a wait that gave up
  int tc_corr, tc_unconv, tc_err;
};

// The mixed-precision kernels of buckets 64 / 96 / 128 (batched_tc.cu).
int batched_tc_bucket(int bucket, int kind, int queue, const int32_t *list, BatchQueues *q,
                      const int32_t *n, const int64_t *offA, const elem_t *A,
                      const int64_t *offv, const elem_t *b, elem_t *x, int32_t *status,
                      int ctas_per_sm);

// Per (size bucket, kind) schedule, chosen by the tuner (tune_batched.py
// writes batched_tune.json, which the library reads at the first batched
// call; compiled-in defaults otherwise): algo 0 = register Gauss-Jordan,
// 1 = blocked LU (buckets 64..128); ctas_per_sm 0 = as many as fit.
struct BatchTune {
  int algo;
  int ctas_per_sm;
};
const BatchTune &batched_tune(int bucket, int kind);

// |v| as a pivot key; NaN loses to every number except in the first row of
// the search, where it wins (mat__iamax keeps its starting element when
// nothing compares greater).
template <typename T>
__device__ __forceinline__ T bkey(T v, bool first) {
  T a = fabs(v);
  if (a != a) return first ? (T)INFINITY : (T)-1;
  return a;
}

// Threads per system: one per row.  NB = 16 packs two systems in a warp.
template <int NB>
struct Tpg {
  static constexpr int v = NB < 16 ? 16 : NB;
};
// Columns per statically unrolled chunk of the row.
template <int NB>
struct Chunk {
  static constexpr int v = NB < 32 ? NB : 32;
};
// Warps (or half warps) per system.
template <int NB>
struct Warps {
  static constexpr int v = NB <= 32 ? 1 : NB / 32;
};

// Lanes of the warp that belong to this thread's system.
template <int NB>
__device__ __forceinline__ unsigned group_mask() {
  if constexpr (NB <= 16)
    return 0xffffu << (threadIdx.x & 16);
  else
    return 0xffffffffu;
}

// Group-wide barrier: a half warp (NB = 16), a warp (NB = 32) or the whole
// CTA (one system per CTA).
template <int NB>
__device__ __forceinline__ void gsync() {
  if constexpr (NB <= 32)
    __syncwarp(group_mask<NB>());
  else
    __syncthreads();
}

// The group barrier as a functor, so a caller that runs several groups of
// more than 32 threads in one CTA can pass a named barrier instead.
template <int NB>
struct GSync {
  __device__ __forceinline__ void operator()() const { gsync<NB>(); }
};
// A named barrier over `count` threads (id 1..15); bar.sync 0 is
// __syncthreads.
struct NamedBar {
  int id, count;
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  }
};

// Row slot: slot[3 + k] = a[k] (k < NB) and slot[NB + 3] = right-hand side,
// so the update's u[j + 1] = slot[j + 4] starts on a 16-byte boundary for
// every 4th (float) or 2nd (double) j and is read with vector loads.
template <int NB>
struct SlotLen {
  static constexpr int v = NB + 4;
};

// Pivot keys: float |a| as an unsigned integer with the same order (see
// fkey), so a warp finds its best candidate with two redux operations; the
// double build compares the values themselves.
template <typename T>
struct PivKey {
  using type = T;
};
template <>
struct PivKey<float> {
  using type = unsigned;
};

// Unsigned key of a float pivot candidate: no candidate 0 < NaN below the top
// row 1 < |a| (its bit pattern + 2; non-negative floats order like their
// bits); a NaN in the top row ranks as +inf, as bkey does.
__device__ __forceinline__ unsigned fkey(float v, bool first) {
  const float a = fabsf(v);
  if (a != a) return first ? 0x7f800002u : 1u;
  return __float_as_uint(a) + 2u;
}

template <typename T, int NB>
struct BatchSmem {
  __align__(16) T slot[2][Warps<NB>::v][SlotLen<NB>::v];  // by step parity
  __align__(16) typename PivKey<T>::type wkey[2][4];        // per warp
  __align__(16) int widx[2][4];
};

template <typename T>
struct VecOf;
template <>
struct VecOf<float> {
  using type = float4;
  static constexpr int w = 4;
  static __device__ __forceinline__ void get(const float *p, float (&o)[4]) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  static __device__ __forceinline__ void put(float *p, const float (&o)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
  }
};
template <>
struct VecOf<double> {
  using type = double2;
  static constexpr int w = 2;
  static __device__ __forceinline__ void get(const double *p, double (&o)[2]) {
    const double2 v = *reinterpret_cast<const double2 *>(p);
    o[0] = v.x; o[1] = v.y;
  }
  static __device__ __forceinline__ void put(double *p, const double (&o)[2]) {
    *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
  }
};

// Write the owned row and its right-hand side into a slot with 16-byte
// stores: slot[3] = a[0], then a[1..NB-1] and the right-hand side at
// slot[4..NB+3], in chunks of Chunk columns -- a chunk is written when it
// holds a live entry (the test shift_update makes before reading it), else
// only the right-hand side, when it falls in the last chunk.
template <typename T, int NB>
__device__ __forceinline__ void put_row(T *slot, const T (&a)[NB], T rb,
                                        int n_live) {
  constexpr int W = VecOf<T>::w;
  constexpr int C = Chunk<NB>::v;
  constexpr int NC = NB / C;
  slot[3] = a[0];
#pragma unroll
  for (int c = 0; c < NC; c++) {
    if (c * C + 1 < n_live) {
#pragma unroll
      for (int g = c * C / W; g < (c + 1) * C / W; g++) {
        T v[W];
#pragma unroll
        for (int q = 0; q < W; q++) {
          const int k = W * g + 1 + q;
          v[q] = k < NB ? a[k] : rb;
        }
        VecOf<T>::put(slot + 4 + W * g, v);
      }
    } else if (c == NC - 1) {
      slot[NB + 3] = rb;
    }
  }
}

// One elimination step in the shifted frame: a[j] <- a[j+1] - u[j+1] * l over
// the chunks that still hold live output columns (j < n_out); entries past
// the live ones are never read into live ones, so partial chunks need no
// masking.  rb <- rb - u_rhs * l.
template <typename T, int NB>
__device__ __forceinline__ void shift_update(T (&a)[NB], T &rb, const T *slot,
                                             T l, int n_out) {
  constexpr int C = Chunk<NB>::v;
  constexpr int W = VecOf<T>::w;
#pragma unroll
  for (int c = 0; c < NB / C; c++) {
    if (c * C < n_out) {
#pragma unroll
      for (int j0 = c * C; j0 < c * C + C; j0 += W) {
        T u[W];
        VecOf<T>::get(slot + j0 + 4, u);
#pragma unroll
        for (int q = 0; q < W; q++) {
          const int j = j0 + q;
          if (j + 1 < NB) a[j] = fma(-u[q], l, a[j + 1]);
        }
      }
    }
  }
  rb = fma(-slot[NB + 3], l, rb);
}

// Solve one system of order n <= NB with the group's NB threads (thread i
// owns row i).  Gauss-Jordan in a shifted register frame: before step K every
// row holds its entries of columns K..n-1 in a[0..n-K-1], so the pivot column
// is always a[0] and every register index is static while the step loop is
// an ordinary loop (compact code).  Step K picks the pivot row, every other
// row eliminates column K (rows above the pivot included, so no back
// substitution is needed), and all rows shift left by one.  At the end the
// row playing logical row r holds x_r * d_r in its right-hand side, d_r its
// pivot.
//
// KIND 0 (general): partial pivoting with mat_plu's rule -- the first
// logical row of max |a| among rows K..n-1, the last column not searched --
// rows trading roles (a logical row index per thread) instead of data.
// Each warp's best candidate stages its row in shared memory before the one
// barrier of the step, so the winner's row is read from its warp's slot.  A
// pivot below eps is not eliminated with (mat_plu skips such columns).
// KIND 1 (SPD): the symmetric matrix is rebuilt from the lower triangle
// (all that mat_chol reads), no row exchanges, and a pivot d_K <= 0 -- the
// Schur-complement diagonal mat_chol tests -- makes the status -1 and leaves
// x untouched.  Returns the status.
template <typename T, int NB, int KIND, class Bar = GSync<NB>>
__device__ int solve_one(const T *__restrict__ A, int n,
                         const T *__restrict__ b, T *__restrict__ x,
                         BatchSmem<T, NB> &sm, int i, T eps, Bar bar = Bar()) {
  const bool act = i < n;
  const int w = NB <= 32 ? 0 : (i >> 5);
  const unsigned gm = group_mask<NB>();
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
  int lr = i;  // logical row played by this thread
  T dg = T(1);
  for (int K = 0; K < n; K++) {
    const int par = K & 1;
    const int live = n - K;  // live entries per row before the step
    int p = K;
    int pw = 0;
    if (KIND == 0 && K < n - 1) {
      const bool cand = act && lr >= K;
      if constexpr (sizeof(T) == 4 && NB >= 32) {
        // warp best by two redux operations on the integer keys: the
        // largest key, then the smallest logical row holding it
        const unsigned key = cand ? fkey(a[0], lr == K) : 0u;
        const unsigned wk = __reduce_max_sync(0xffffffffu, key);
        const unsigned wi = __reduce_min_sync(
            0xffffffffu, (cand && key == wk) ? (unsigned)lr : 0x7fffffffu);
        // lane 0 publishes the warp's best as (key, row << 2 | warp); the
        // rows are distinct, so the smallest code among the best keys is
        // the smallest row and names its warp's slot
        if ((i & 31) == 0) {
          sm.wkey[par][w] = wk;
          sm.widx[par][w] = (int)((wi << 2) | (unsigned)w);
        }
        if (cand && (unsigned)lr == wi) put_row<T, NB>(sm.slot[par][w], a, rb, live);
        bar();
        if constexpr (Warps<NB>::v == 1) {
          p = (int)wi;
        } else {
          const int lane = i & 31;
          const unsigned ck = lane < Warps<NB>::v ? sm.wkey[par][lane] : 0u;
          const unsigned ci = lane < Warps<NB>::v ? (unsigned)sm.widx[par][lane] : 0xffffffffu;
          const unsigned bk = __reduce_max_sync(0xffffffffu, ck);
          const unsigned bi = __reduce_min_sync(0xffffffffu, ck == bk ? ci : 0xffffffffu);
          p = (int)(bi >> 2);
          pw = (int)(bi & 3u);
        }
      } else {
        T key = cand ? bkey(a[0], lr == K) : (T)-2;
        int idx = cand ? lr : 0x7fffffff;
#pragma unroll
        for (int off = (NB <= 16 ? 8 : 16); off > 0; off >>= 1) {
          const T ok = __shfl_xor_sync(gm, key, off);
          const int oi = __shfl_xor_sync(gm, idx, off);
          if (ok > key || (ok == key && oi < idx)) {
            key = ok;
            idx = oi;
          }
        }
        // every warp publishes its best key (-2: no candidate left in it)
        if ((i & 31) == 0) {
          sm.wkey[par][w] = key;
          sm.widx[par][w] = idx;
        }
        if (cand && lr == idx) put_row<T, NB>(sm.slot[par][w], a, rb, live);
        bar();
        p = sm.widx[par][0];
        if constexpr (Warps<NB>::v > 1) {
          T bk = sm.wkey[par][0];
#pragma unroll
          for (int q = 1; q < Warps<NB>::v; q++) {
            const T kq = sm.wkey[par][q];
            const int iq = sm.widx[par][q];
            if (kq > bk || (kq == bk && iq < p)) {
              bk = kq;
              p = iq;
              pw = q;
            }
          }
        }
      }
    } else {
      // the pivot is logical row K itself
      if (act && lr == K) put_row<T, NB>(sm.slot[par][0], a, rb, live);
      bar();
    }
    const T *u = sm.slot[par][pw];
    const T piv = u[3];
    if (KIND == 1 && piv <= T(0)) return -1;  // NaN passes, as in mat_chol
    const int old = lr;
    const bool is_piv = act && old == p;
    if (is_piv) {
      lr = K;
      dg = a[0];
    } else if (act && old == K) {
      lr = p;
    }
    // one code path for every row: the pivot row (and every row when the
    // pivot is too small to eliminate with) shifts with multiplier 0, which
    // leaves its entries unchanged (live entries are finite)
    const bool elim = KIND == 1 || !(fabs(piv) < eps);
    const T l = (act && elim && !is_piv) ? a[0] * (T(1) / piv) : T(0);
    shift_update<T, NB>(a, rb, u, l, live - 1);
  }
  if (act && lr >= 0 && lr < n) x[lr] = rb / dg;  // lr < n by construction
  return 0;
}

// General systems, diagonal pivots first (KIND 2): the same Gauss-Jordan
// steps with logical row K as the pivot of step K, so a step needs no pivot
// search -- the row's owner stages it, one barrier, every row eliminates.
// Each row below K checks that partial pivoting would have kept row K (its
// key no larger than row K's; equal keys go to the smaller row, K), and if
// any row of the system ever would have won, the system is solved again by
// solve_one with the search.  Otherwise the pivot sequence is partial
// pivoting's and every operation is the one solve_one performs, so x is
// the same either way.  Diagonally dominant systems never fall back.
template <typename T>
__device__ __forceinline__ auto spec_key(T v, bool first) {
  if constexpr (sizeof(T) == 4)
    return fkey(v, first);
  else
    return bkey(v, first);
}

// The fallback as a call of its own, so its register frame does not add to
// the diagonal-first loop's.
template <typename T, int NB, class Bar>
__device__ __noinline__ int solve_pivoted(const T *__restrict__ A, int n,
                                          const T *__restrict__ b, T *__restrict__ x,
                                          BatchSmem<T, NB> &sm, int i, T eps, Bar bar) {
  return solve_one<T, NB, 0, Bar>(A, n, b, x, sm, i, eps, bar);
}

template <typename T, int NB, class Bar = GSync<NB>>
__device__ int solve_diag_first(const T *__restrict__ A, int n,
                                const T *__restrict__ b, T *__restrict__ x,
                                BatchSmem<T, NB> &sm, int i, T eps, Bar bar = Bar()) {
  const bool act = i < n;
  T a[NB];
  T rb = act ? b[i] : T(0);
#pragma unroll
  for (int j = 0; j < NB; j++) a[j] = (act && j < n) ? A[i + (int64_t)j * n] : T(0);
  T dg = T(1);
  bool beaten = false;
  for (int K = 0; K < n; K++) {
    const int par = K & 1;
    const int live = n - K;
    if (act && i == K) {
      put_row<T, NB>(sm.slot[par][0], a, rb, live);
      sm.slot[par][0][2] = T(1) / a[0];  // the pivot's reciprocal, divided once
    }
    bar();
    const T *u = sm.slot[par][0];
    const T piv = u[3];
    // the last column is not searched (mat_plu)
    if (act && i > K && K < n - 1 && spec_key(a[0], false) > spec_key(piv, true))
      beaten = true;
    const bool is_piv = act && i == K;
    if (is_piv) dg = a[0];
    const bool elim = !(fabs(piv) < eps);
    const T l = (act && elim && !is_piv) ? a[0] * u[2] : T(0);
    shift_update<T, NB>(a, rb, u, l, live - 1);
  }
  // did partial pivoting pick another row anywhere?
  bool any;
  if constexpr (Warps<NB>::v == 1) {
    any = __any_sync(group_mask<NB>(), beaten);
  } else {
    const bool wany = __any_sync(0xffffffffu, beaten);
    if ((i & 31) == 0) sm.widx[0][i >> 5] = wany ? 1 : 0;
    bar();
    any = false;
#pragma unroll
    for (int w = 0; w < Warps<NB>::v; w++) any = any || sm.widx[0][w] != 0;
    bar();  // the flags are read before the next system reuses them
  }
  if (!any) {
    if (act) x[i] = rb / dg;
    return 0;
  }
  return solve_pivoted<T, NB, Bar>(A, n, b, x, sm, i, eps, bar);
}

// ---------------------------------------------------------------------------
// SPD systems: LDL^T elimination on the lower triangle (all that mat_chol
// reads), thread i owning row i, no exchanges.  Before step K row i >= K
// holds A^(K)[i][K..i] in a[0..i-K] (shifted frame, pivot column in a[0]).
// Step K: every row i >= K publishes its a[0] -- column K of the Schur
// complement, d_K = the pivot at its head -- and row K its right-hand side
// y_K; after the group barrier every row i > K takes l = a[0]/d_K and
// a[m] <- a[m+1] - l * col_K[m+1] over its i-K live entries, y_i -= l*y_K.
// A pivot d_K <= 0 (mat_chol's test, NaN passes) makes the status -1 and
// leaves x untouched.  A warp whose rows are all done takes no updates.
// The published columns stay in shared memory (triangular, each column's
// entries 16-byte aligned for the vector loads) and give the back
// substitution x_K = (y_K - sum_{i>K} col_K[i-K] x_i) * (1/d_K), one unknown
// per barrier, every row folding each new x into its own sum.
template <int NB>
struct SpdCols {
  // sum over K of roundup4(NB - K + 3), plus the reach of one chunk past
  // the last column's entries
  static constexpr int v = [] {
    int s = 0;
    for (int K = 0; K < NB; K++) s += (NB - K + 3 + 3) / 4 * 4;
    return s + 40;
  }();
};

template <typename T, int NB>
struct SpdSmem {
  __align__(16) T cols[SpdCols<NB>::v];
  T ys[NB];
  T xs[NB];
};

template <typename T, int NB, class Bar = GSync<NB>>
__device__ int solve_spd(const T *__restrict__ A, int n,
                         const T *__restrict__ b, T *__restrict__ x,
                         SpdSmem<T, NB> &sm, int i, Bar bar = Bar()) {
  constexpr int C = Chunk<NB>::v;
  constexpr int W = VecOf<T>::w;
  constexpr int GW = NB < 32 ? NB : 32;  // rows of one warp (half warp)
  const bool act = i < n;
  T a[NB];
  T rb = act ? b[i] : T(0);
#pragma unroll
  for (int j = 0; j < NB; j++) a[j] = (act && j <= i && j < n) ? A[i + (int64_t)j * n] : T(0);
  // last row of this thread's warp (half warp) that belongs to the system
  const int wlast = ((i | (GW - 1)) < n - 1 ? (i | (GW - 1)) : n - 1);
  T rdg = T(1);  // 1 / this row's pivot
  int myoff = 0;
  int off = 0;
  for (int K = 0; K < n; K++) {
    T *col = sm.cols + off;
    if (act && i >= K) col[3 + (i - K)] = a[0];
    if (i == K) {
      sm.ys[K] = rb;
      myoff = off;
      col[2] = T(1) / a[0];  // the pivot's reciprocal, divided once
    }
    bar();
    const T d = col[3];
    if (d <= T(0)) return -1;  // NaN passes, as in mat_chol
    const T rd = col[2];
    if (i == K) rdg = rd;
    const int n_out = wlast - K;  // the warp's longest remaining row
    if (n_out > 0) {
      const T l = (act && i > K) ? a[0] * rd : T(0);
#pragma unroll
      for (int c = 0; c < NB / C; c++) {
        if (c * C < n_out) {
#pragma unroll
          for (int j0 = c * C; j0 < c * C + C; j0 += W) {
            T u[W];
            VecOf<T>::get(col + j0 + 4, u);
#pragma unroll
            for (int q = 0; q < W; q++) {
              const int j = j0 + q;
              if (j + 1 < NB) a[j] = fma(-u[q], l, a[j + 1]);
            }
          }
        }
      }
      rb = fma(-sm.ys[K], l, rb);
    }
    off += (n - K + 3 + 3) / 4 * 4;
  }
  // back substitution, rb = y_i: one unknown per barrier from the last up,
  // every earlier row folding it into its sum
  T xi = T(0);
  for (int K = n - 1; K >= 0; K--) {
    if (i == K) {
      xi = rb * rdg;
      sm.xs[K] = xi;
    }
    bar();
    if (act && i < K) rb = fma(-sm.cols[myoff + 3 + (K - i)], sm.xs[K], rb);
  }
  if (act) x[i] = xi;
  return 0;
}

// Resident CTAs per SM asked of the register allocator for the two largest
// buckets (the row itself takes NB registers): 3 x 128 and 4 x 96 threads.
template <int NB>
struct MinCtas {
  static constexpr int v = NB == 128 ? 3 : NB == 96 ? 4 : 1;
};

// Persistent: every group pulls systems of its queue until it is empty.
template <typename T, int NB, int GROUPS, int KIND>
__global__ void __launch_bounds__(Tpg<NB>::v *GROUPS, MinCtas<NB>::v)
    batched_kernel(int queue, const int32_t *__restrict__ list,
                   BatchQueues *q, const int32_t *__restrict__ nvec,
                   const int64_t *__restrict__ offA, const T *__restrict__ A,
                   const int64_t *__restrict__ offv, const T *__restrict__ b,
                   T *__restrict__ x, int32_t *__restrict__ status, T eps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using Smem = typename std::conditional<KIND == 1, SpdSmem<T, NB>, BatchSmem<T, NB>>::type;
  Smem *smem = reinterpret_cast<Smem *>(smem_raw);
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
    int st;
    if constexpr (KIND == 1)
      st = solve_spd<T, NB>(A + offA[s], n, b + offv[s], x + offv[s], smem[g], i);
    else if constexpr (KIND == 2)
      st = solve_diag_first<T, NB>(A + offA[s], n, b + offv[s], x + offv[s],
                                   smem[g], i, eps);
    else
      st = solve_one<T, NB, KIND>(A + offA[s], n, b + offv[s], x + offv[s],
                                  smem[g], i, eps);
    if (i == 0) status[s] = st;
    gsync<NB>();
  }
}

template <typename T, int NB, int GROUPS, int KIND>
int launch_batched_queue(int queue, const int32_t *list, BatchQueues *q,
                         const int32_t *n, const int64_t *offA, const T *A,
                         const int64_t *offv, const T *b, T *x,
                         int32_t *status, T eps, int ctas_per_sm = 0) {
  auto k = batched_kernel<T, NB, GROUPS, KIND>;
  constexpr int threads = Tpg<NB>::v * GROUPS;
  using Smem = typename std::conditional<KIND == 1, SpdSmem<T, NB>, BatchSmem<T, NB>>::type;
  const size_t smem = sizeof(Smem) * GROUPS;
  static bool attr = false;
  if (!attr) {
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    attr = true;
  }
  int per_sm = 0;
  MGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem));
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  if (per_sm < 1) per_sm = 1;
  const int grid = ctx()->sms * per_sm;
  static const char *names[2][5] = {
      {"batched_lu_16", "batched_lu_32", "batched_lu_64", "batched_lu_96", "batched_lu_128"},
      {"batched_spd_16", "batched_spd_32", "batched_spd_64", "batched_spd_96", "batched_spd_128"}};
  KtScope kt(names[KIND == 1][NB <= 16 ? 0 : NB <= 32 ? 1 : NB <= 64 ? 2 : NB <= 96 ? 3 : 4], 0.0, 0.0);
  k<<<grid, threads, smem, ctx()->stream>>>(queue, list, q, n, offA, A, offv, b,
                                            x, status, eps);
  MGB_LAUNCHED("batched_solve");
  return 0;
}

// One entry point per (bucket, kind), each in its own translation unit
// batched_nb<NB>_<lu|chol>.cu so the kernels compile in parallel.
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
