// Partial-pivot LU (mat_plu / mat_solve's factorisation), GB300 layout.
//
// Reference algorithm: mat__plu_blocked_ (mat.h:4201-4289) -- right-looking,
// 24-column panels, pivot = first index of max |a| (mat__iamax,
// mat.h:1247-1262), pivots with |a| < MAT_DEFAULT_EPSILON swapped in but not
// divided by (mat.h:4235-4236), reciprocal-multiply column scaling
// (mat.h:4238-4240), delayed row swaps on the trailing columns, TRSM for U12
// and a GEMM trailing update.
//
// GB300 design:
//  * Panel (24 columns, the reference's block, so the pivot-skip rule acts on
//    exactly the same column groups): ONE launch of a thread-block cluster of
//    up to 16 CTAs.  The panel rows are split across the CTAs' shared memory
//    (up to ~3.5 MB across 16 SMs).  Per column: each thread scans its own rows
//    (warp-shuffle arg-max with first-index tie-break), each CTA publishes its
//    candidate row and the current row k into every CTA's shared memory
//    (DSMEM stores), one hardware cluster barrier, then every CTA picks the
//    winner, swaps, scales and updates its own rows.  Two barriers per column
//    (one CTA-local, one cluster-wide); no global-memory round trip.
//  * Row swaps (laswp): one warp turns a block's swap sequence into a net
//    row mapping (touched rows -> source rows); every CTA then gathers the
//    touched rows of 32 columns into shared memory with all loads in flight
//    and writes them back permuted.
//  * U12 = L11^{-1} A12: one thread per right-hand-side column, the column in
//    registers and L11 in shared memory (no block barriers).
//  * Outer blocks of 96 columns with look-ahead: the panel chain runs on a
//    high-priority stream while the previous block's trailing GEMM runs on
//    the library stream; events order the two.
#include <cooperative_groups.h>
#include <limits.h>

#include <vector>

#include "internal.cuh"
#include "lp_pack.cuh"

namespace cg = cooperative_groups;

namespace mgb {

constexpr int kPanelThreads = 512;
constexpr int kPanelWarps = kPanelThreads / 32;
constexpr int kRefBlock = 24;  // MAT_PLU_BLOCK_SIZE, mat.h:4196
constexpr int kOuterBlock = 96;   // plain path (SIMT trailing GEMM)
constexpr int kOuterBlockLp = 128;  // tensor-core path (K of tc_gemm)
constexpr int kSmemMax = 227 * 1024;

template <typename T>
__device__ __forceinline__ T piv_key(T v, bool first) {
  // Reproduces mat__amax_scalar + mat__iamax on NaNs: a NaN at the first
  // position wins (max becomes NaN, no index compares equal, index 0 is
  // returned); NaNs elsewhere never win.
  T a = fabs(v);
  if (a != a) return first ? (T)INFINITY : (T)-1;
  return a;
}

template <typename T>
__device__ __forceinline__ bool better(T k1, int i1, T k2, int i2) {
  return k1 > k2 || (k1 == k2 && i1 < i2);
}

template <typename T>
static size_t panel_smem(int cs, int w, int rpc) {
  size_t t = (size_t)w * rpc + kPanelWarps + 2 * cs + 2 * (size_t)cs * w +
             2 * (size_t)w;
  return t * sizeof(T) + (kPanelWarps + 2 * cs) * sizeof(int);
}

// Factor rows [k0, n) x columns [k0, k0+w) of A in place.  ipiv[k0+kk] gets
// the global row swapped into row k0+kk.  One cluster; CTA c holds panel rows
// [c*rpc, (c+1)*rpc).  Thread tid owns local rows tid, tid+512, ...
template <typename T>
__global__ void __launch_bounds__(kPanelThreads, 1)
    lu_panel_kernel(T *__restrict__ A, int64_t lda, int64_t n, int64_t k0,
                    int w, int rpc, int32_t *__restrict__ ipiv, T eps) {
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int c = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t m = n - k0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *P = (T *)smem_raw;
  T *wkey = P + (size_t)w * rpc;
  T *xkey = wkey + kPanelWarps;
  T *xval = xkey + 2 * CS;
  T *kval = xval + 2 * (size_t)CS * w;
  int *widx = (int *)(kval + 2 * w);
  int *xidx = widx + kPanelWarps;

  const int64_t rbase = (int64_t)c * rpc;
  for (int r = tid; r < rpc; r += kPanelThreads) {
    const int64_t pr = rbase + r;
    for (int j = 0; j < w; j++)
      P[(size_t)j * rpc + r] = pr < m ? A[(k0 + pr) + (k0 + j) * lda] : T(0);
  }

  for (int kk = 0; kk < w; kk++) {
    const int buf = kk & 1;
    // 1. arg-max of |P[kk][r]| over my rows with panel row >= kk
    T bk = (T)-2;
    int bi = INT_MAX;
    for (int r = tid; r < rpc; r += kPanelThreads) {
      const int64_t pr = rbase + r;
      if (pr >= kk && pr < m) {
        T key = piv_key(P[(size_t)kk * rpc + r], pr == kk);
        if (better(key, (int)pr, bk, bi)) {
          bk = key;
          bi = (int)pr;
        }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      T ok = __shfl_down_sync(0xffffffffu, bk, off);
      int oi = __shfl_down_sync(0xffffffffu, bi, off);
      if (better(ok, oi, bk, bi)) {
        bk = ok;
        bi = oi;
      }
    }
    if (lane == 0) {
      wkey[warp] = bk;
      widx[warp] = bi;
    }
    __syncthreads();
    T ck = wkey[0];
    int ci = widx[0];
#pragma unroll
    for (int q = 1; q < kPanelWarps; q++)
      if (better(wkey[q], widx[q], ck, ci)) {
        ck = wkey[q];
        ci = widx[q];
      }
    // 2. publish this CTA's candidate row, and row kk if it lives here
    const bool own_k = (kk >= rbase && kk < rbase + rpc);
    const int nval = CS * w;
    const int total = nval + CS + (own_k ? nval : 0);
    for (int t = tid; t < total; t += kPanelThreads) {
      if (t < nval) {
        const int q = t / w, j = t % w;
        T v = (ci != INT_MAX) ? P[(size_t)j * rpc + (ci - rbase)] : T(0);
        T *dst = cluster.map_shared_rank(xval, q);
        dst[((size_t)buf * CS + c) * w + j] = v;
      } else if (t < nval + CS) {
        const int q = t - nval;
        T *dk = cluster.map_shared_rank(xkey, q);
        int *di = cluster.map_shared_rank(xidx, q);
        dk[buf * CS + c] = ck;
        di[buf * CS + c] = ci;
      } else {
        const int u = t - nval - CS;
        const int q = u / w, j = u % w;
        T *dst = cluster.map_shared_rank(kval, q);
        dst[(size_t)buf * w + j] = P[(size_t)j * rpc + (kk - rbase)];
      }
    }
    cluster.sync();
    // 3. winner over the cluster (every thread, same answer)
    int wc = 0;
    T gk = xkey[buf * CS];
    int gi = xidx[buf * CS];
    for (int q = 1; q < CS; q++)
      if (better(xkey[buf * CS + q], xidx[buf * CS + q], gk, gi)) {
        gk = xkey[buf * CS + q];
        gi = xidx[buf * CS + q];
        wc = q;
      }
    const T *u = xval + ((size_t)buf * CS + wc) * w;
    const T *kv = kval + (size_t)buf * w;
    const int p = gi;
    if (c == 0 && tid == 0) ipiv[k0 + kk] = (int32_t)(k0 + p);
    // 4. swap rows kk and p (only the owning threads touch them)
    if (p != kk) {
      if (p >= rbase && p < rbase + rpc && (int)((p - rbase) % kPanelThreads) == tid)
        for (int j = 0; j < w; j++) P[(size_t)j * rpc + (p - rbase)] = kv[j];
      if (own_k && (int)((kk - rbase) % kPanelThreads) == tid)
        for (int j = 0; j < w; j++) P[(size_t)j * rpc + (kk - rbase)] = u[j];
    }
    // 5. scale column kk and rank-1 update of the panel's later columns
    const T piv = u[kk];
    if (!(fabs(piv) < eps)) {
      const T inv = T(1) / piv;
      for (int r = tid; r < rpc; r += kPanelThreads) {
        const int64_t pr = rbase + r;
        if (pr > kk && pr < m) {
          const T l = P[(size_t)kk * rpc + r] * inv;
          P[(size_t)kk * rpc + r] = l;
          for (int j = kk + 1; j < w; j++)
            P[(size_t)j * rpc + r] = fma(-u[j], l, P[(size_t)j * rpc + r]);
        }
      }
    }
  }

  for (int r = tid; r < rpc; r += kPanelThreads) {
    const int64_t pr = rbase + r;
    if (pr < m)
      for (int j = 0; j < w; j++) A[(k0 + pr) + (k0 + j) * lda] = P[(size_t)j * rpc + r];
  }
}

// A float pivot key as an unsigned integer with the same order: the special
// keys -3 (empty) < -2 (no candidate) < -1 (NaN below the top) map to 0, 1,
// 2, and |a| >= 0 (+inf for a NaN at the top) to its bit pattern + 4
// (non-negative floats order like their bit patterns).
__device__ __forceinline__ unsigned ukey(float k) {
  return k >= 0.f ? __float_as_uint(k) + 4u : (k == -1.f ? 2u : k == -2.f ? 1u : 0u);
}

// Warp-wide best (key, index): largest key, then smallest index (two redux
// operations); every lane gets the winner's key code and index.
__device__ __forceinline__ void warp_best(unsigned uk, int idx, unsigned &bk,
                                          int &bi) {
  bk = __reduce_max_sync(0xffffffffu, uk);
  const unsigned mi = __reduce_min_sync(0xffffffffu, uk == bk ? (unsigned)idx : 0xffffffffu);
  bi = (int)mi;
}

// Lane holding the best of a warp's float candidates (largest key, then
// smallest index) when the candidates' indices increase with the lane within
// each of two ranges, [.., split) before [split, ..): a single max
// reduction and two ballots instead of a second (index) reduction.
__device__ __forceinline__ int first_max_lane(unsigned uk, int idx, int split) {
  const unsigned ub = __reduce_max_sync(0xffffffffu, uk);
  const unsigned h0 = __ballot_sync(0xffffffffu, uk == ub && idx < split);
  const unsigned h1 = __ballot_sync(0xffffffffu, uk == ub);
  return __ffs(h0 ? h0 : h1) - 1;
}

// Best (key, index) of cnt <= 32 candidates in shared memory, reduced across
// the warp (every lane gets the result and the winner's slot).  Ties between
// real candidates cannot happen (their indices are distinct).
// The best of cnt <= 32 float candidates given as (index << 32 | key bits)
// words, whose indices increase with the slot.
__device__ __forceinline__ void pick_first_ki(const unsigned long long *ki, int cnt, float &bk,
                                              int &bi, int &bw) {
  const int lane = threadIdx.x & 31;
  const unsigned long long w = lane < cnt ? ki[lane] : 0ull;
  const float k = lane < cnt ? __uint_as_float((unsigned)w) : -3.f;
  const int i = lane < cnt ? (int)(unsigned)(w >> 32) : INT_MAX;
  bw = first_max_lane(ukey(k), i, INT_MAX);
  bi = __shfl_sync(0xffffffffu, i, bw);
  bk = __shfl_sync(0xffffffffu, k, bw);
}

// The same for float candidates whose indices increase with the slot within
// [.., split) and within [split, ..).
__device__ __forceinline__ void pick_first(const float *keys, const int *idxs, int cnt,
                                           int split, float &bk, int &bi, int &bw) {
  const int lane = threadIdx.x & 31;
  const float k = lane < cnt ? keys[lane] : -3.f;
  const int i = lane < cnt ? idxs[lane] : INT_MAX;
  bw = first_max_lane(ukey(k), i, split);
  bi = __shfl_sync(0xffffffffu, i, bw);
  bk = __shfl_sync(0xffffffffu, k, bw);
}

template <typename T>
__device__ __forceinline__ void pick_best(const T *keys, const int *idxs,
                                          int cnt, T &bk, int &bi, int &bw) {
  const int lane = threadIdx.x & 31;
  if constexpr (sizeof(T) == 4) {
    const T k = lane < cnt ? keys[lane] : (T)-3;
    const int i = lane < cnt ? idxs[lane] : INT_MAX;
    unsigned ub;
    warp_best(ukey(k), i, ub, bi);
    const unsigned hit = __ballot_sync(0xffffffffu, lane < cnt && i == bi && ukey(k) == ub);
    bw = hit ? __ffs(hit) - 1 : 0;
    bk = __shfl_sync(0xffffffffu, k, bw);
    return;
  }
  T k = lane < cnt ? keys[lane] : (T)-3;
  int i = lane < cnt ? idxs[lane] : INT_MAX;
  int w = lane;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const T ok = __shfl_xor_sync(0xffffffffu, k, off);
    const int oi = __shfl_xor_sync(0xffffffffu, i, off);
    const int ow = __shfl_xor_sync(0xffffffffu, w, off);
    if (better(ok, oi, k, i)) {
      k = ok;
      i = oi;
      w = ow;
    }
  }
  bk = k;
  bi = i;
  bw = w;
}

// Register-resident panel for the reference's 24-column width: thread tid of
// CTA c owns panel rows c*rpc + tid + r*NT (r < R), all 24 columns of each in
// registers; the column loop is unrolled so every register index is static.
// Per column: arg-max over owned rows, warp shuffles, each warp's candidate
// row staged in shared memory, CTA-level pick, DSMEM publication of the CTA
// candidate (and of row kk) to every CTA by st.async completing on the
// receiver's own mbarrier (no cluster barrier per column), swap, scale,
// rank-1 update in registers.
constexpr int kW = kRefBlock;

template <typename T, int NT>
struct RegPanelSmem {
  __align__(16) T wrow[NT / 32][kW];
  __align__(16) T krow[kW];
  T wkey[NT / 32];
  int widx[NT / 32];
  __align__(16) T xval[2][16][kW];
  __align__(8) T xkey[2][16];
  int xidx[2][16];
  // float: key bits and index in one 8-byte word (one message, not two)
  __align__(8) unsigned long long xki[2][16];
  __align__(16) T kval[2][kW];
  // exchange barriers by step parity: the arm (with the step's expected
  // bytes from the other CTAs), one arrival per local warp once its share of
  // the local copy is stored, and the other CTAs' st.async bytes
  __align__(8) uint64_t xbar[2];
};

// Device flag: a panel exchange gave up waiting (never expected; a lost
// transfer ends the wait instead of hanging the GPU).
__device__ int g_lu_wait_err = 0;

namespace xch {
__device__ __forceinline__ uint32_t saddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// the same shared-memory offset in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa(uint32_t a, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}
__device__ __forceinline__ void fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void arm(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)),
               "r"(bytes)
               : "memory");
}
// Bounded wait for the phase with the given parity (acquire at cluster
// scope: the bytes were written by other CTAs' st.async).  Gives up after
// about 2^25 cycles (~16 ms; a column's exchange takes microseconds), or at
// once when an earlier wait has already given up, so a lost transfer costs
// one timeout, not one per column.
__device__ __forceinline__ bool wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = saddr(bar);
  long long t0 = 0;
  for (int i = 0;; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 15) == 15) {
      const long long now = clock64();
      if (t0 == 0)
        t0 = now;
      else if (now - t0 > (1ll << 25))
        return false;
      if (*reinterpret_cast<volatile int *>(&g_lu_wait_err)) return false;
    }
  }
}
__device__ __forceinline__ void put16(uint32_t dst, const void *src, uint32_t bar) {
  const uint4 v = *reinterpret_cast<const uint4 *>(src);
  asm volatile(
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];"
      ::"r"(dst), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void put4(uint32_t dst, uint32_t v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];"
               ::"r"(dst), "r"(v), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void put8(uint32_t dst, uint64_t v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];"
               ::"r"(dst), "l"(v), "r"(bar)
               : "memory");
}
}  // namespace xch

// Bytes a CTA receives from the other CTAs per column: each one's candidate
// row, key and index, plus row kk when another CTA owns it (a CTA's own
// contributions are plain shared-memory stores).
template <typename T>
__host__ __device__ constexpr uint32_t xch_bytes(int cs, bool kk_remote) {
  return (uint32_t)((cs - 1) * (kW * sizeof(T) + sizeof(T) + sizeof(int)) +
                    (kk_remote ? kW * sizeof(T) : 0));
}

// Exchange set-up at the start of a panel kernel: both barriers initialised
// (one arrival for the arm plus one per warp) and armed for the first two
// columns (owner0/owner1: CTAs holding their rows kk), then one cluster
// barrier so no CTA sends before every receiver's barriers exist.
template <typename T, int NT>
__device__ __forceinline__ void xch_setup(RegPanelSmem<T, NT> &sm, cg::cluster_group &cluster,
                                          int cs, int c, int owner0, int owner1) {
  if (threadIdx.x == 0) {
    xch::init(&sm.xbar[0], 1 + NT / 32);
    xch::init(&sm.xbar[1], 1 + NT / 32);
    xch::fence_init();
    xch::arm(&sm.xbar[0], xch_bytes<T>(cs, owner0 != c));
    xch::arm(&sm.xbar[1], xch_bytes<T>(cs, owner1 != c));
  }
  cluster.sync();
}

// A 24-value row to / from 16-byte aligned shared memory (vector accesses
// for float).
template <typename T>
__device__ __forceinline__ void row_put(T *dst, const T (&v)[kW]) {
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int j = 0; j < kW; j += 4)
      *reinterpret_cast<float4 *>(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
  } else {
#pragma unroll
    for (int j = 0; j < kW; j++) dst[j] = v[j];
  }
}
template <typename T>
__device__ __forceinline__ void row_get(const T *src, T (&v)[kW]) {
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int j = 0; j < kW; j += 4) {
      const float4 f = *reinterpret_cast<const float4 *>(src + j);
      v[j] = f.x; v[j + 1] = f.y; v[j + 2] = f.z; v[j + 3] = f.w;
    }
  } else {
#pragma unroll
    for (int j = 0; j < kW; j++) v[j] = src[j];
  }
}

// Net row maps of a swap sequence, kept up to date one pivot at a time by
// one warp (defined with SwapMap below): the panel's (every CTA) and, in one
// CTA, the whole block's.
struct SwapMap;
__device__ __forceinline__ void swap_map_reset(SwapMap &map, int64_t k0, int nk);
__device__ __forceinline__ void swap_map_step(SwapMap &map, int64_t k0, int nk, int i,
                                              int32_t P);
struct MapSink {
  SwapMap *panel;  // this panel's map (null: none kept)
  SwapMap *block;  // the block's map (null: none kept here)
  int64_t kb;      // the block's first row
  int bw;          // the block's width
};

// The 24-column elimination of a register-resident panel (rows [k0, n) of
// A, columns [k0, k0+24)): thread tid of CTA c owns panel rows prow[r]
// (panel-relative, -1 = none) in a[r][*].  ipiv[k0+kk] (CTA 0) and, when
// spiv is given, spiv[kk] (every CTA, shared memory) get the global pivot row.
//
// Rotating frame: before column kk every row holds column kk in a[r][0],
// columns kk+1..23 in a[r][1..23-kk] and its finished columns 0..kk-1 in
// a[r][24-kk..23]; each step rotates the row left by one (live entries get
// the rank-1 update on the way, the new multiplier lands in a[r][23]), so
// after 24 steps every row is back in natural order.  The column loop is an
// ordinary loop over static register indices -- one copy of the step in the
// instruction stream instead of 24 -- and the arithmetic is exactly that of
// the unrolled form (the same FMAs on the same operands).
// step: this kernel's running column count (the exchange barriers' phase),
// nsteps: its total columns (no barrier is armed past the last).
// maps (may be null): the panel's net row map and the block's, built by the
// last warp while it waits for each column's exchange (pivot kk-1 during
// column kk's wait, the last pivot after the loop); complete once the
// caller synchronises the CTA.
template <typename T, int R, int NT>
__device__ __forceinline__ void reg_panel_columns(
    T (&a)[R][kW], const int (&prow)[R], RegPanelSmem<T, NT> &sm,
    cg::cluster_group &cluster, int c, int CS, int rbase, int rpc, int mrows,
    int64_t k0, int32_t *__restrict__ ipiv, int32_t *spiv, T eps, int &step,
    int nsteps,
    const MapSink *maps = nullptr) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = NT / 32;
  (void)cluster;
  const bool mapper = maps && warp == NW - 1;
  if (mapper) swap_map_reset(*maps->panel, k0, kW);
  int32_t pprev = 0;
  auto map_pivot = [&](int i) {
    swap_map_step(*maps->panel, k0, kW, i, pprev);
    if (maps->block)
      swap_map_step(*maps->block, maps->kb, maps->bw, (int)(k0 - maps->kb) + i, pprev);
  };
  // Exchange pieces (16-byte pieces of a row; per receiver: the candidate
  // row, its key and index, and row kk when this CTA owns it).  In float
  // every thread below CS*PER sends one fixed piece to one fixed receiver
  // every column, so its destinations (both parities) are mapped once here.
  constexpr int NV = kW * (int)sizeof(T) / 16;
  constexpr int PER = 2 * NV + 1;  // float: row, key+index, row kk
  constexpr bool kFixed = sizeof(T) == 4 && NT >= 16 * PER;
  const int sq = tid / PER, se = tid % PER;
  const bool sender = kFixed && sq < CS;
  uint32_t sdst0 = 0, sdst1 = 0, sbar0 = 0, sbar1 = 0;
  if (sender && sq != c) {
    auto dst_of = [&](int b) -> uint32_t {
      if (se < NV) return xch::mapa(xch::saddr(&sm.xval[b][c][0]), sq) + 16 * se;
      if (se == NV) return xch::mapa(xch::saddr(&sm.xki[b][c]), sq);
      return xch::mapa(xch::saddr(&sm.kval[b][0]), sq) + 16 * (se - NV - 1);
    };
    sdst0 = dst_of(0);
    sdst1 = dst_of(1);
    sbar0 = xch::mapa(xch::saddr(&sm.xbar[0]), sq);
    sbar1 = xch::mapa(xch::saddr(&sm.xbar[1]), sq);
    // never expected: a misaligned barrier is flagged (the receiver's wait
    // then gives up), never used
    if ((sbar0 | sbar1) & 7u) g_lu_wait_err = 2;
  }
#pragma unroll 1
  for (int kk = 0; kk < kW; kk++, step++) {
    const int buf = step & 1;
    // arm the other barrier for the next column before this CTA sends this
    // column's data (no CTA can send column step+1 before receiving ours);
    // its previous phase (column step-1) completed at the last wait.  The
    // next column's row kk lives in CTA (kk+1)/rpc, or in CTA 0 when it
    // opens the next panel.
    if (tid == 0 && step >= 1 && step + 1 < nsteps) {
      const int nown = kk + 1 < kW ? (kk + 1) / rpc : 0;
      xch::arm(&sm.xbar[buf ^ 1], xch_bytes<T>(CS, nown != c));
    }
    T bk = (T)-2;
    int bi = INT_MAX;
#pragma unroll
    for (int r = 0; r < R; r++)
      if (prow[r] >= kk) {
        const T key = piv_key(a[r][0], prow[r] == kk);
        if (better(key, prow[r], bk, bi)) { bk = key; bi = prow[r]; }
      }
    // the rows of this CTA: [rbase, rbase+NT) in thread order, then (R = 2)
    // [rbase+NT, ..) in thread order, so within each range the index grows
    // with the lane and with the warp
    const int split = rbase + NT;
    constexpr bool kOrdered = sizeof(T) == 4 && R <= 2;
    if constexpr (kOrdered) {
      const int wl = first_max_lane(ukey(bk), bi, split);
      bi = __shfl_sync(0xffffffffu, bi, wl);
      bk = __shfl_sync(0xffffffffu, bk, wl);
    } else if constexpr (sizeof(T) == 4) {
      unsigned ub;
      warp_best(ukey(bk), bi, ub, bi);
      bk = __shfl_sync(0xffffffffu, bk, __ffs(__ballot_sync(0xffffffffu, ukey(bk) == ub)) - 1);
    } else {
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const T ok = __shfl_xor_sync(0xffffffffu, bk, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (better(ok, oi, bk, bi)) { bk = ok; bi = oi; }
      }
    }
    // every lane now holds the warp's best; its owner stages the row
#pragma unroll
    for (int r = 0; r < R; r++) {
      if (prow[r] >= 0 && prow[r] == bi) row_put<T>(&sm.wrow[warp][0], a[r]);
      if (prow[r] == kk) row_put<T>(&sm.krow[0], a[r]);
    }
    if (lane == 0) { sm.wkey[warp] = bk; sm.widx[warp] = bi; }
    __syncthreads();
    T ck;
    int ci, cw;
    if constexpr (kOrdered)
      pick_first(sm.wkey, sm.widx, NW, split, ck, ci, cw);
    else
      pick_best<T>(sm.wkey, sm.widx, NW, ck, ci, cw);
    const bool own_k = (kk >= rbase && kk < rbase + rpc);
    // 16-byte pieces of a row; per receiver: the candidate row, its key and
    // index, and row kk when this CTA owns it.  Other CTAs get st.async
    // (completing bytes on their barrier), this CTA plain stores; every warp
    // then arrives on the local barrier, so its completion also means every
    // local sender has read its staging row
    const T *srow = ci != INT_MAX ? &sm.wrow[cw][0] : nullptr;
    if constexpr (kFixed) {
      const unsigned long long kiw =
          ((unsigned long long)(unsigned)ci << 32) | __float_as_uint((float)ck);
      if (sender && (se < NV + 1 || own_k)) {
        if (sq == c) {
          if (se < NV) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (srow) v = *reinterpret_cast<const uint4 *>(reinterpret_cast<const char *>(srow) + 16 * se);
            *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(&sm.xval[buf][c][0]) + 16 * se) = v;
          } else if (se == NV) {
            sm.xki[buf][c] = kiw;
          } else {
            const int o = 16 * (se - NV - 1);
            *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(&sm.kval[buf][0]) + o) =
                *reinterpret_cast<const uint4 *>(reinterpret_cast<const char *>(&sm.krow[0]) + o);
          }
        } else if (!((sbar0 | sbar1) & 7u)) {
          const uint32_t dst = buf ? sdst1 : sdst0, rbar = buf ? sbar1 : sbar0;
          if (se < NV) {
            if (srow) {
              xch::put16(dst, reinterpret_cast<const char *>(srow) + 16 * se, rbar);
            } else {
              const uint4 z = make_uint4(0, 0, 0, 0);
              xch::put16(dst, &z, rbar);
            }
          } else if (se == NV) {
            xch::put8(dst, kiw, rbar);
          } else {
            xch::put16(dst, reinterpret_cast<const char *>(&sm.krow[0]) + 16 * (se - NV - 1), rbar);
          }
        }
      }
    }
    // otherwise: one loop over all pieces (double rows need more threads)
    if constexpr (!kFixed) {
      const int per = NV + 2 + (own_k ? NV : 0);
      const uint32_t lbar = xch::saddr(&sm.xbar[buf]);
      for (int t = tid; t < CS * per; t += NT) {
        const int q = t / per, e = t % per;
        if (q == c) {
          if (e < NV) {
            uint4 v = make_uint4(0, 0, 0, 0);
            if (srow) v = *reinterpret_cast<const uint4 *>(reinterpret_cast<const char *>(srow) + 16 * e);
            *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(&sm.xval[buf][c][0]) + 16 * e) = v;
          } else if (e == NV) {
            sm.xkey[buf][c] = ck;
          } else if (e == NV + 1) {
            sm.xidx[buf][c] = ci;
          } else {
            const int o = 16 * (e - NV - 2);
            *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(&sm.kval[buf][0]) + o) =
                *reinterpret_cast<const uint4 *>(reinterpret_cast<const char *>(&sm.krow[0]) + o);
          }
          continue;
        }
        const uint32_t rbar = xch::mapa(lbar, q);
        if (rbar & 7u) {  // never expected: a misaligned barrier is flagged, not used
          g_lu_wait_err = 2;
          continue;
        }
        if (e < NV) {
          const uint32_t dst = xch::mapa(xch::saddr(&sm.xval[buf][c][0]), q) + 16 * e;
          if (srow) {
            xch::put16(dst, reinterpret_cast<const char *>(srow) + 16 * e, rbar);
          } else {
            const uint4 z = make_uint4(0, 0, 0, 0);
            xch::put16(dst, &z, rbar);
          }
        } else if (e == NV) {
          const uint32_t dst = xch::mapa(xch::saddr(&sm.xkey[buf][c]), q);
          if constexpr (sizeof(T) == 4)
            xch::put4(dst, __float_as_uint((float)ck), rbar);
          else
            xch::put8(dst, (uint64_t)__double_as_longlong((double)ck), rbar);
        } else if (e == NV + 1) {
          xch::put4(xch::mapa(xch::saddr(&sm.xidx[buf][c]), q), (uint32_t)ci, rbar);
        } else {
          const uint32_t dst = xch::mapa(xch::saddr(&sm.kval[buf][0]), q) + 16 * (e - NV - 2);
          xch::put16(dst, reinterpret_cast<const char *>(&sm.krow[0]) + 16 * (e - NV - 2), rbar);
        }
      }
    }
    __syncwarp();
    if (lane == 0) xch::arrive(&sm.xbar[buf]);
    if (mapper && kk > 0) map_pivot(kk - 1);
    const bool got = xch::wait(&sm.xbar[buf], (uint32_t)(step >> 1) & 1u);
    if (!got) g_lu_wait_err = 1;
    T gk;
    int p, wc;
    // CTA q's candidate lies in [q*rpc, (q+1)*rpc): indices grow with q
    if constexpr (kFixed) {
      float gkf;
      pick_first_ki(sm.xki[buf], CS, gkf, p, wc);
      gk = (T)gkf;
    } else if constexpr (sizeof(T) == 4) {
      pick_first(sm.xkey[buf], sm.xidx[buf], CS, INT_MAX, gk, p, wc);
    } else {
      pick_best<T>(sm.xkey[buf], sm.xidx[buf], CS, gk, p, wc);
    }
    // A wait that gave up leaves the exchange slots stale (or never written):
    // take no pivot from them.  The step then keeps row kk in place and
    // eliminates nothing, so every index written below stays in [k0, n) and
    // the kernels queued behind this one see a valid (if meaningless) swap
    // sequence; the host reports MATGB_ERR_TIMEOUT after its next sync.
    if (!got || p < kk || p >= mrows) {
      p = kk;
      wc = c;
    }
    if (c == 0 && tid == 0) ipiv[k0 + kk] = (int32_t)(k0 + p);
    if (spiv && tid == 0) spiv[kk] = (int32_t)(k0 + p);
    pprev = (int32_t)(k0 + p);
    const T *u = &sm.xval[buf][wc][0];
    const T *kv = &sm.kval[buf][0];
    if (p != kk) {
#pragma unroll
      for (int r = 0; r < R; r++) {
        if (prow[r] == p) {
#pragma unroll
          for (int j = 0; j < kW; j++) a[r][j] = kv[j];
        } else if (prow[r] == kk) {
#pragma unroll
          for (int j = 0; j < kW; j++) a[r][j] = u[j];
        }
      }
    }
    const T piv = u[0];
    const bool elim = got && !(fabs(piv) < eps);
    const T inv = elim ? T(1) / piv : T(0);
    const int live = kW - 1 - kk;  // columns right of kk
    T uj[kW];
    row_get<T>(u, uj);
#pragma unroll
    for (int r = 0; r < R; r++) {
      const bool upd = elim && prow[r] > kk;
      const T l = upd ? a[r][0] * inv : a[r][0];
#pragma unroll
      for (int j = 0; j < kW - 1; j++)
        a[r][j] = (upd && j < live) ? fma(-uj[j + 1], l, a[r][j + 1]) : a[r][j + 1];
      a[r][kW - 1] = l;
    }
  }
  if (mapper) map_pivot(kW - 1);
}

template <typename T, int R, int NT>
__global__ void __launch_bounds__(NT, 1)
    lu_panel_reg_kernel(T *__restrict__ A, int64_t lda, int64_t n, int64_t k0,
                        int rpc, int32_t *__restrict__ ipiv, T eps) {
  __shared__ RegPanelSmem<T, NT> sm;
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int c = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const int m = (int)(n - k0);
  const int rbase = c * rpc;
  int prow[R];
  T a[R][kW];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int lr = tid + r * NT;
    prow[r] = (lr < rpc && rbase + lr < m) ? rbase + lr : -1;
#pragma unroll
    for (int j = 0; j < kW; j++)
      a[r][j] = prow[r] >= 0 ? A[(k0 + prow[r]) + (k0 + j) * lda] : T(0);
  }
  xch_setup<T, NT>(sm, cluster, CS, c, 0, 1 / rpc);
  int step = 0;
  reg_panel_columns<T, R, NT>(a, prow, sm, cluster, c, CS, rbase, rpc, m, k0,
                              ipiv, nullptr, eps, step, kW);
#pragma unroll
  for (int r = 0; r < R; r++)
    if (prow[r] >= 0)
#pragma unroll
      for (int j = 0; j < kW; j++) A[(k0 + prow[r]) + (k0 + j) * lda] = a[r][j];
}

// ---- row swaps ----------------------------------------------------------------
// Net effect of the swap sequence ipiv[k1..k2) (global row indices, each
// ipiv[k] >= k) on rows: after it, row pos[t] holds the original row src[t]
// for t < cnt; every other row is unchanged.  Built by one warp in shared
// memory: positions [k1,k2) are indexed directly, pivot rows beyond k2 are
// found by a warp-wide search.
constexpr int kSwapMax = 160;  // pivots per swap block (the fused path uses 144)

struct SwapMap {
  int32_t pos[2 * kSwapMax];
  int32_t src[2 * kSwapMax];
  int32_t piv[kSwapMax];  // the pivot sequence, loaded once in parallel
  int cnt;
};

__device__ void build_swap_map(SwapMap &sm, const int32_t *__restrict__ ipiv,
                               int64_t k1, int64_t k2) {
  const int lane = threadIdx.x & 31;
  const int nk = (int)(k2 - k1);
  for (int i = lane; i < nk; i += 32) {
    sm.pos[i] = (int32_t)(k1 + i);
    sm.src[i] = (int32_t)(k1 + i);
    sm.piv[i] = ipiv[k1 + i];  // all loads in flight at once, not one per step
  }
  __syncwarp();
  int nx = 0;  // extra rows (>= k2) at pos[nk .. nk+nx)
  for (int i = 0; i < nk; i++) {
    const int32_t k = (int32_t)(k1 + i);
    const int32_t p = sm.piv[i];
    if (p <= k) continue;  // p < k: never written by a factorisation; no swap
    int slot;
    if (p < k2) {
      slot = p - (int32_t)k1;
    } else {
      int found = -1;
      for (int base = 0; base < nx; base += 32) {
        const int t = base + lane;
        unsigned m = __ballot_sync(0xffffffffu, t < nx && sm.pos[nk + t] == p);
        if (m) {
          found = base + __ffs(m) - 1;
          break;
        }
      }
      if (found < 0) {
        if (lane == 0) {
          sm.pos[nk + nx] = p;
          sm.src[nk + nx] = p;
        }
        __syncwarp();
        found = nx++;
      }
      slot = nk + found;
    }
    if (lane == 0) {
      int32_t t = sm.src[i];
      sm.src[i] = sm.src[slot];
      sm.src[slot] = t;
    }
    __syncwarp();
  }
  if (lane == 0) sm.cnt = nk + nx;
}

// The same map kept up to date one pivot at a time by one warp (the fused
// block's panels): reset for the nk pivots starting at row k0, then pivot i
// (global row P) applied -- the steps of build_swap_map's loop.
__device__ __forceinline__ void swap_map_reset(SwapMap &map, int64_t k0, int nk) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < nk; i += 32) {
    map.pos[i] = (int32_t)(k0 + i);
    map.src[i] = (int32_t)(k0 + i);
  }
  if (lane == 0) map.cnt = nk;
  __syncwarp();
}
__device__ __forceinline__ void swap_map_step(SwapMap &map, int64_t k0, int nk, int i,
                                              int32_t P) {
  const int lane = threadIdx.x & 31;
  // P < k0 + i never comes from a completed exchange (the pick is over rows
  // at or below the step); it is treated as no swap rather than indexing
  // the map with a negative slot
  if (P <= (int32_t)(k0 + i)) return;
  int slot;
  if (P < (int32_t)(k0 + nk)) {
    slot = P - (int32_t)k0;
  } else {
    // rows beyond the first nk sit at [nk, cnt), at most nk of them
    const int cnt = map.cnt;
    int found = -1;
    for (int base = nk; base < cnt; base += 32) {
      const unsigned hit =
          __ballot_sync(0xffffffffu, base + lane < cnt && map.pos[base + lane] == P);
      if (hit) {
        found = base + __ffs(hit) - 1;
        break;
      }
    }
    if (found >= 0) {
      slot = found;
    } else {
      slot = cnt;
      if (lane == 0) {
        map.pos[cnt] = P;
        map.src[cnt] = P;
        map.cnt = cnt + 1;
      }
    }
  }
  if (lane == 0) {
    const int32_t t = map.src[i];
    map.src[i] = map.src[slot];
    map.src[slot] = t;
  }
  __syncwarp();
}

// The map is built once per swap block by one warp (swap_map_kernel) into a
// small device ring; the swap kernel's CTAs read it.
__global__ void swap_map_kernel(const int32_t *__restrict__ ipiv, int64_t k1,
                                int64_t k2, SwapMap *__restrict__ out) {
  __shared__ SwapMap sm;
  build_swap_map(sm, ipiv, k1, k2);
  __syncwarp();
  const int cnt = sm.cnt;
  for (int i = threadIdx.x; i < cnt; i += 32) {
    out->pos[i] = sm.pos[i];
    out->src[i] = sm.src[i];
  }
  if (threadIdx.x == 0) out->cnt = cnt;
}

// Apply the row mapping to columns [c0,c1) and [c2,c3) and, on CTA 0, to the
// permutation vector.  One warp per column at a time (8 warps, 32 columns per
// CTA), lanes across the map entries: the rows of the block [k1,k2) are
// contiguous in a column, so that half of every gather/scatter coalesces; a
// column is read whole into registers before it is written.
constexpr int kSwapCols = 32;

// BUILD: few CTAs (a swap inside a block column) -- warp 0 of every CTA
// builds the map itself, saving the extra launch; otherwise it comes from
// swap_map_kernel.
template <typename T, bool BUILD>
__global__ void __launch_bounds__(256)
    laswp_kernel(T *__restrict__ A, int64_t lda, int64_t c0, int64_t c1,
                 int64_t c2, int64_t c3, const SwapMap *__restrict__ map,
                 const int32_t *__restrict__ ipiv, int64_t k1, int64_t k2,
                 int32_t *__restrict__ perm, int cpb = kSwapCols) {
  constexpr int RPL = 2 * kSwapMax / 32;  // map entries per lane
  __shared__ SwapMap sm;
  if (BUILD) {
    if (threadIdx.x < 32) build_swap_map(sm, ipiv, k1, k2);
  } else {
    const int c = __ldg(&map->cnt);
    for (int r = threadIdx.x; r < c; r += 256) {
      sm.pos[r] = __ldg(&map->pos[r]);
      sm.src[r] = __ldg(&map->src[r]);
    }
    if (threadIdx.x == 0) sm.cnt = c;
  }
  __syncthreads();
  const int cnt = sm.cnt;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t src[RPL], pos[RPL];
#pragma unroll
  for (int q = 0; q < RPL; q++) {
    const int r = lane + 32 * q;
    src[q] = r < cnt ? sm.src[r] : 0;
    pos[q] = r < cnt ? sm.pos[r] : 0;
  }
  const int64_t na = c1 - c0, nb = c3 - c2;
  for (int cc = warp; cc < cpb; cc += 8) {
    const int64_t t = (int64_t)blockIdx.x * cpb + cc;
    if (t >= na + nb) break;
    T *colp = A + (t < na ? c0 + t : c2 + (t - na)) * lda;
    T v[RPL];
#pragma unroll
    for (int q = 0; q < RPL; q++)
      if (lane + 32 * q < cnt) v[q] = colp[src[q]];
    __syncwarp();
#pragma unroll
    for (int q = 0; q < RPL; q++)
      if (lane + 32 * q < cnt) colp[pos[q]] = v[q];
  }
  if (blockIdx.x == 0 && perm) {
    // the permutation vector: one warp, same scheme
    if (warp == 0) {
      int32_t pv[RPL];
#pragma unroll
      for (int q = 0; q < RPL; q++)
        if (lane + 32 * q < cnt) pv[q] = perm[src[q]];
      __syncwarp();
#pragma unroll
      for (int q = 0; q < RPL; q++)
        if (lane + 32 * q < cnt) perm[pos[q]] = pv[q];
    }
  }
}

// Ring of device swap maps: the panel stream and the main stream each use
// one slot at a time, and a slot is rewritten only several blocks later,
// after stream order has retired its readers.
constexpr int kSwapRing = 16;
static SwapMap *g_swap_ring = nullptr;
static int g_swap_next = 0;

static SwapMap *swap_ring_slot() {
  if (!g_swap_ring && cudaMalloc(&g_swap_ring, kSwapRing * sizeof(SwapMap)) != cudaSuccess) {
    cudaGetLastError();
    g_swap_ring = nullptr;
    return nullptr;
  }
  SwapMap *m = g_swap_ring + g_swap_next;
  g_swap_next = (g_swap_next + 1) % kSwapRing;
  return m;
}

template <typename T>
int laswp_t(T *A, int64_t lda, int64_t c0, int64_t c1, int64_t c2, int64_t c3,
            const int32_t *ipiv, int64_t k1, int64_t k2, int32_t *perm,
            SwapMap *keep) {
  const int64_t ncol = (c1 - c0) + (c3 - c2);
  if (k2 <= k1 || (ncol <= 0 && !perm && !keep)) return 0;
  if (k2 - k1 > kSwapMax) return set_error(MATGB_ERR_ARG, "laswp: block > %d", kSwapMax);
  if (!g_swap_ring) MGB_CUDA(cudaMalloc(&g_swap_ring, kSwapRing * sizeof(SwapMap)));
  // keep: the block's net map is also wanted later (deferred swaps)
  SwapMap *map = keep ? keep : g_swap_ring + g_swap_next;
  if (!keep) g_swap_next = (g_swap_next + 1) % kSwapRing;
  int64_t blocks = (ncol + kSwapCols - 1) / kSwapCols;
  if (blocks < 1) blocks = 1;
  KtScope kt("laswp", 0.0, 4.0 * (k2 - k1) * ncol * sizeof(T));
  if (blocks <= 8 && !keep) {
    laswp_kernel<T, true><<<(unsigned)blocks, 256, 0, ctx()->stream>>>(
        A, lda, c0, c1, c2, c3, nullptr, ipiv, k1, k2, perm);
  } else {
    swap_map_kernel<<<1, 32, 0, ctx()->stream>>>(ipiv, k1, k2, map);
    MGB_LAUNCHED("swap_map");
    laswp_kernel<T, false><<<(unsigned)blocks, 256, 0, ctx()->stream>>>(
        A, lda, c0, c1, c2, c3, map, ipiv, k1, k2, perm);
  }
  MGB_LAUNCHED("laswp");
  return 0;
}

// The same swaps from a net map already on the device (the fused block
// kernel writes its block's): no map build in the swap stream.
template <typename T>
static int laswp_map(T *A, int64_t lda, int64_t c0, int64_t c1, int64_t c2, int64_t c3,
                     const SwapMap *map, int32_t *perm, int64_t npiv) {
  const int64_t ncol = (c1 - c0) + (c3 - c2);
  if (ncol <= 0 && !perm) return 0;
  // few columns (the look-ahead's): one column per warp, so the column
  // loads of every warp are in flight at once
  const int cpb = ncol <= 1024 ? 8 : kSwapCols;
  int64_t blocks = (ncol + cpb - 1) / cpb;
  if (blocks < 1) blocks = 1;
  KtScope kt("laswp", 0.0, 4.0 * npiv * ncol * sizeof(T));
  laswp_kernel<T, false><<<(unsigned)blocks, 256, 0, ctx()->stream>>>(
      A, lda, c0, c1, c2, c3, map, nullptr, 0, 0, perm, cpb);
  MGB_LAUNCHED("laswp");
  return 0;
}

// ---- deferred row swaps on the factored columns --------------------------
// A right-looking factorisation never reads the columns of a finished block
// again, so the swaps of later blocks' pivots can reach those columns at the
// end, in one pass, instead of block by block: for column block b, rows
// [ke_b, n) are gathered through G_b = s_{b+1} o s_{b+2} o ... (s_k: block
// k's net swap map as a gather, row pos[t] <- row src[t]).  The same moves as
// swapping block by block, so L is identical; the pass reads and writes each
// column once, coalesced, instead of touching scattered rows per block.
// G_b for every block, built backwards in one CTA with a dense map in shared
// memory (n entries).
__global__ void __launch_bounds__(1024)
    swap_compose_kernel(const SwapMap *__restrict__ maps, int nblk, int64_t n,
                        int64_t nb, int32_t *__restrict__ G) {
  extern __shared__ int32_t dmap[];
  const int tid = threadIdx.x;
  for (int64_t i = tid; i < n; i += 1024) dmap[i] = (int32_t)i;
  __syncthreads();
  for (int b = nblk - 2; b >= 0; b--) {
    const SwapMap &m = maps[b + 1];
    const int cnt = m.cnt;
    for (int t = tid; t < cnt; t += 1024) dmap[m.pos[t]] = m.src[t];
    __syncthreads();
    const int64_t r0 = (int64_t)(b + 1) * nb;      // rows below block b
    const int64_t r1 = (int64_t)(b + 2) * nb;      // rows below block b + 1
    for (int64_t i = r0 + tid; i < n; i += 1024) {
      const int32_t g1 = (i < r1 || b + 1 == nblk - 1) ? (int32_t)i : G[(int64_t)(b + 1) * n + i];
      G[(int64_t)b * n + i] = dmap[g1];
    }
    __syncthreads();
    for (int t = tid; t < cnt; t += 1024) dmap[m.pos[t]] = m.pos[t];
    __syncthreads();
  }
}

// One CTA per column of the first nblk-1 blocks: the column's rows below its
// block into shared memory (coalesced), then written back through G_b.
template <typename T>
__global__ void __launch_bounds__(256)
    left_gather_kernel(T *__restrict__ A, int64_t lda, int64_t n, int64_t nb,
                       const int32_t *__restrict__ G) {
  extern __shared__ __align__(16) unsigned char lg_raw[];
  T *col = reinterpret_cast<T *>(lg_raw);
  const int64_t j = blockIdx.x;
  const int64_t b = j / nb;
  const int64_t r0 = (b + 1) * nb;
  T *cp = A + j * lda;
  for (int64_t i = r0 + threadIdx.x; i < n; i += 256) col[i - r0] = cp[i];
  __syncthreads();
  const int32_t *g = G + b * n;
  for (int64_t i = r0 + threadIdx.x; i < n; i += 256) {
    const int64_t s = g[i];
    if (s >= r0 && s < n) cp[i] = col[s - r0];  // always true: later swaps stay below the block
  }
}

template <typename T>
static int apply_deferred_swaps(T *A, int64_t lda, int64_t n, int64_t nb, int nblk,
                                const SwapMap *maps, int32_t *G) {
  cudaStream_t st = ctx()->stream;
  const size_t dsm = (size_t)n * sizeof(int32_t);
  static bool attr = false;
  if (!attr) {
    MGB_CUDA(cudaFuncSetAttribute(swap_compose_kernel,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemMax));
    MGB_CUDA(cudaFuncSetAttribute(left_gather_kernel<T>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemMax));
    attr = true;
  }
  {
    KtScope kt("swap_compose", 0.0, 8.0 * n * nblk);
    swap_compose_kernel<<<1, 1024, dsm, st>>>(maps, nblk, n, nb, G);
    MGB_LAUNCHED("swap_compose");
  }
  const int64_t ncols = (int64_t)(nblk - 1) * nb;
  KtScope kt("left_gather", 0.0, 2.0 * sizeof(T) * (double)ncols * (n - nb) / 2.0);
  left_gather_kernel<T><<<(unsigned)ncols, 256, (size_t)(n - nb) * sizeof(T), st>>>(
      A, lda, n, nb, G);
  MGB_LAUNCHED("left_gather");
  return 0;
}

// ---- fused block factorisation (mixed-precision path) --------------------
// One cluster launch factors the whole outer block A[kb:n, kb:kb+bw) (bw a
// multiple of 24, the block held in L2 between phases): for each 24-column
// panel -- the register panel elimination (reg_panel_columns), its row swaps
// applied to the block's other columns, U12 = L11^-1 A12 for the block
// columns right of the panel, and the rank-24 update of the rows below from
// the L21 rows still in registers.  A cluster barrier separates the phases;
// data written by another CTA is read with ld.global.cg (L2), so no stale L1
// line is ever used.  The panels keep the reference's 24-column width and its
// pivot-skip rule (eps), so the plain float LU uses it too.
constexpr int kFusedMaxBw = 144;

// 24 consecutive values from 16-byte aligned shared memory.
template <typename T>
struct VecLoad {
  static __device__ __forceinline__ void get24(const T *p, T (&o)[kW]) {
#pragma unroll
    for (int k = 0; k < kW; k++) o[k] = p[k];
  }
};
template <>
struct VecLoad<float> {
  static __device__ __forceinline__ void get24(const float *p, float (&o)[kW]) {
#pragma unroll
    for (int k = 0; k < kW; k += 4) {
      const float4 v = *reinterpret_cast<const float4 *>(p + k);
      o[k] = v.x; o[k + 1] = v.y; o[k + 2] = v.z; o[k + 3] = v.w;
    }
  }
};

template <typename T, int NT>
struct FusedSmem {
  RegPanelSmem<T, NT> ps;
  SwapMap map;   // the current panel's net row map
  SwapMap bmap;  // the block's (CTA 0)
  int32_t spiv[kW];
  T L11[kW][kW + 1];
  __align__(16) T U12t[kFusedMaxBw - kW][kW];  // U12 transposed: k contiguous
};

template <typename T, int R, int NT>
__global__ void __launch_bounds__(NT, 1)
    lu_block_fused_kernel(T *__restrict__ A, int64_t lda, int64_t n,
                          int64_t kb, int bw, int32_t *__restrict__ ipiv, T eps,
                          unsigned *__restrict__ amax_l, SwapMap *__restrict__ bmap_out) {
  __shared__ FusedSmem<T, NT> sm;
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int c = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NWARP = NT / 32;
  const int np = bw / kW;
  // the block's net row map (for the swaps of the columns outside the
  // block) is built by CTA 0's last warp along with the panels' maps
  const bool keep_block = bmap_out && c == 0;
  const MapSink sink = {&sm.map, keep_block ? &sm.bmap : nullptr, kb, bw};
  if (keep_block && warp == NWARP - 1) swap_map_reset(sm.bmap, kb, bw);
  {
    const int rpc0 = (int)((n - kb) + CS - 1) / CS;  // the first panel's rows per CTA
    xch_setup<T, NT>(sm.ps, cluster, CS, c, 0, 1 / rpc0);
  }
  int step = 0;
  for (int pn = 0; pn < np; pn++) {
    const int64_t k0 = kb + (int64_t)pn * kW;
    const int m = (int)(n - k0);
    const int rpc = (m + CS - 1) / CS;
    const int rbase = c * rpc;
    int prow[R];
    T a[R][kW];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int lr = tid + r * NT;
      prow[r] = (lr < rpc && rbase + lr < m) ? rbase + lr : -1;
#pragma unroll
      for (int j = 0; j < kW; j++)
        a[r][j] = prow[r] >= 0 ? __ldcg(&A[(k0 + prow[r]) + (k0 + j) * lda]) : T(0);
    }
    reg_panel_columns<T, R, NT>(a, prow, sm.ps, cluster, c, CS, rbase, rpc, m, k0,
                                ipiv, sm.spiv, eps, step, np * kW, &sink);
#pragma unroll
    for (int r = 0; r < R; r++)
      if (prow[r] >= 0)
#pragma unroll
        for (int j = 0; j < kW; j++) A[(k0 + prow[r]) + (k0 + j) * lda] = a[r][j];
    if (amax_l) {
      // an upper bound of max |L21| (the tensor-core operand's FP16 scale):
      // the panel's multipliers of every row below its diagonal block -- the
      // later panels' swaps only permute those rows, so L21 (the rows below
      // the block at the end) is a subset; NaN ignored as in amax_kernel
      float mx = 0.f;
#pragma unroll
      for (int r = 0; r < R; r++)
        if (prow[r] >= kW)
#pragma unroll
          for (int j = 0; j < kW; j++) mx = fmaxf(mx, fabsf((float)a[r][j]));
      for (int off = 16; off; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
      if (lane == 0 && mx > 0.f) atomicMax(amax_l, __float_as_uint(mx));
    }
    // the panel's swaps on the block's other columns: [kb, k0) and
    // [k0+24, kb+bw); CTA c takes every CS-th of them, one warp per column
    // (the map was built during the panel)
    __syncthreads();
    const int nleft = (int)(k0 - kb), nright = bw - (pn + 1) * kW;
    {
      const int cnt = sm.map.cnt;
      for (int t = c + CS * warp; t < nleft + nright; t += CS * NWARP) {
        const int64_t col = t < nleft ? kb + t : k0 + kW + (t - nleft);
        T *colp = A + col * lda;
        T v[2 * kW / 32 + 1];
#pragma unroll
        for (int q = 0; q < 2 * kW / 32 + 1; q++) {
          const int r = lane + 32 * q;
          if (r < cnt) v[q] = __ldcg(&colp[sm.map.src[r]]);
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 2 * kW / 32 + 1; q++) {
          const int r = lane + 32 * q;
          if (r < cnt) colp[sm.map.pos[r]] = v[q];
        }
      }
    }
    if (nright <= 0) break;  // the block's last panel: nothing to its right
    cluster.sync();
    // U12 = L11^-1 A12 for the right columns (rows k0..k0+23), one warp per
    // column: lane l holds row l, x_k broadcast by shuffle
    for (int e = tid; e < kW * kW; e += NT) {
      const int i = e % kW, j = e / kW;
      sm.L11[i][j] = __ldcg(&A[(k0 + i) + (k0 + j) * lda]);
    }
    __syncthreads();
    for (int t = c + CS * warp; t < nright; t += CS * NWARP) {
      T *colp = A + (k0 + kW + t) * lda + k0;
      T x = lane < kW ? __ldcg(&colp[lane]) : T(0);
#pragma unroll
      for (int k = 0; k < kW - 1; k++) {
        const T xk = __shfl_sync(0xffffffffu, x, k);
        if (lane > k && lane < kW) x = fma(-sm.L11[lane][k], xk, x);
      }
      if (lane < kW) colp[lane] = x;
    }
    cluster.sync();
    // rank-24 update of the rows below the panel, right columns, a group of
    // columns at a time with the next group's L2 loads in flight
    for (int e = tid; e < kW * nright; e += NT) {
      const int i = e % kW, j = e / kW;
      sm.U12t[j][i] = __ldcg(&A[(k0 + i) + (k0 + kW + j) * lda]);
    }
    __syncthreads();
    constexpr int JB = R == 1 ? 8 : 4;  // columns per group (registers allow 8 at one row)
    T *base = A + (k0 + kW) * lda + k0;
    auto load_cols = [&](T (&v)[R][JB], int j0) {
#pragma unroll
      for (int r = 0; r < R; r++)
#pragma unroll
        for (int jj = 0; jj < JB; jj++)
          v[r][jj] = (prow[r] >= kW && j0 + jj < nright)
                         ? __ldcg(&base[(int64_t)(j0 + jj) * lda + prow[r]])
                         : T(0);
    };
    auto update_cols = [&](T (&v)[R][JB], int j0) {
#pragma unroll
      for (int jj = 0; jj < JB; jj++) {
        if (j0 + jj < nright) {
          T uj[kW];
          VecLoad<T>::get24(&sm.U12t[j0 + jj][0], uj);
#pragma unroll
          for (int r = 0; r < R; r++)
#pragma unroll
            for (int k = 0; k < kW; k++) v[r][jj] = fma(-a[r][k], uj[k], v[r][jj]);
        }
      }
#pragma unroll
      for (int r = 0; r < R; r++)
#pragma unroll
        for (int jj = 0; jj < JB; jj++)
          if (prow[r] >= kW && j0 + jj < nright)
            base[(int64_t)(j0 + jj) * lda + prow[r]] = v[r][jj];
    };
    T v0[R][JB], v1[R][JB];
    load_cols(v0, 0);
    for (int j0 = 0; j0 < nright; j0 += 2 * JB) {
      load_cols(v1, j0 + JB);
      update_cols(v0, j0);
      if (j0 + 2 * JB < nright) load_cols(v0, j0 + 2 * JB);
      update_cols(v1, j0 + JB);
    }
    cluster.sync();
  }
  if (keep_block && warp == NWARP - 1) {
    const int cnt = sm.bmap.cnt;
    for (int i = lane; i < cnt; i += 32) {
      bmap_out->pos[i] = sm.bmap.pos[i];
      bmap_out->src[i] = sm.bmap.src[i];
    }
    if (lane == 0) bmap_out->cnt = cnt;
  }
}

// ---- U12 = L11^{-1} A12 with L11 unit lower (TB x TB) ----------------------
// A warp solves CPW right-hand-side columns at once: lane l holds rows l,
// l+32, ... of each in registers, L11 sits in shared memory; step k
// broadcasts each column's x_k by a shuffle and every lane updates its rows
// below k -- per column the reference's axpy order (mat.h:4264-4271); the
// CPW columns' chains interleave and share each L11 load.  Loads and stores
// of a column are coalesced.  The CTAs stride over the columns (at most two
// per SM), so that each stages L11 once for many columns; the staging copies
// 16 bytes at a time when the columns start on 16-byte boundaries.
template <typename T, int TB, int CPW>
__global__ void __launch_bounds__(256)
    trsm_unit_warp_kernel(const T *__restrict__ L, int64_t ldl,
                          T *__restrict__ B, int64_t ldb, int64_t ncols,
                          unsigned *__restrict__ amax) {
  constexpr int RPL = (TB + 31) / 32;
  constexpr int VE = 16 / (int)sizeof(T);  // elements per 16-byte copy
  constexpr int LS = TB + VE;               // staged column stride (16-byte)
  static_assert(TB % VE == 0, "16-byte columns of L11");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *Ls = (T *)smem_raw;  // Ls[k*LS + i] = L(i, k)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // L11 staged by asynchronous copies, a warp per column
  if (ldl % VE == 0 && (reinterpret_cast<uintptr_t>(L) & 15) == 0) {
    for (int k = warp; k < TB; k += 8)
      for (int c = lane; c < TB / VE; c += 32) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&Ls[k * LS + VE * c]);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst),
                     "l"(&L[VE * c + (int64_t)k * ldl])
                     : "memory");
      }
  } else {
    for (int k = warp; k < TB; k += 8)
      for (int i = lane; i < TB; i += 32) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&Ls[k * LS + i]);
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(dst),
                     "l"(&L[i + (int64_t)k * ldl]), "n"(sizeof(T))
                     : "memory");
      }
  }
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  float m = 0.f;  // max |U12| over the warp's columns (float builds)
  const int64_t step = (int64_t)gridDim.x * 8 * CPW;
  for (int64_t c0 = ((int64_t)blockIdx.x * 8 + warp) * CPW; c0 < ncols; c0 += step) {
    T x[CPW][RPL];
#pragma unroll
    for (int c = 0; c < CPW; c++) {
      const T *b = B + (c0 + c) * ldb;
#pragma unroll
      for (int r = 0; r < RPL; r++) {
        const int i = lane + 32 * r;
        x[c][r] = (c0 + c < ncols && i < TB) ? b[i] : T(0);
      }
    }
#pragma unroll
    for (int k = 0; k < TB - 1; k++) {
      T xk[CPW];
#pragma unroll
      for (int c = 0; c < CPW; c++) xk[c] = __shfl_sync(0xffffffffu, x[c][k / 32], k % 32);
#pragma unroll
      for (int r = k / 32; r < RPL; r++) {
        const int i = lane + 32 * r;
        if (i > k && i < TB) {
          const T l = Ls[k * LS + i];
#pragma unroll
          for (int c = 0; c < CPW; c++) x[c][r] = fma(-l, xk[c], x[c][r]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < CPW; c++) {
      if (c0 + c >= ncols) break;
      T *b = B + (c0 + c) * ldb;
#pragma unroll
      for (int r = 0; r < RPL; r++) {
        const int i = lane + 32 * r;
        if (i > 0 && i < TB) b[i] = x[c][r];
        // the FP16 scale of the tensor-core operand; NaN ignored as in
        // amax_kernel
        if (sizeof(T) == 4 && i < TB) m = fmaxf(m, fabsf((float)x[c][r]));
      }
    }
  }
  if constexpr (sizeof(T) == 4) {
    if (amax) {
      for (int off = 16; off; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
      if (lane == 0 && m > 0.f) atomicMax(amax, __float_as_uint(m));
    }
  }
}

template <typename T, int TB>
static int launch_trsm_warp(int64_t ncols, const T *L, int64_t ldl, T *B,
                            int64_t ldb, unsigned *amax) {
  // four columns per warp once every warp of two CTAs per SM has that many
  const int64_t cap = 2 * (int64_t)ctx()->sms;
  const bool wide = ncols >= cap * 8 * 4;
  auto k = wide ? trsm_unit_warp_kernel<T, TB, 4> : trsm_unit_warp_kernel<T, TB, 1>;
  const size_t smem = (size_t)TB * (TB + 16 / sizeof(T)) * sizeof(T);
  static bool attr[2] = {false, false};
  if (!attr[wide]) {
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    attr[wide] = true;
  }
  int64_t blocks = (ncols + 8 * (wide ? 4 : 1) - 1) / (8 * (wide ? 4 : 1));
  if (blocks > cap) blocks = cap;
  KtScope kt("trsm_lu", (double)TB * TB * ncols, (double)sizeof(T) * 2.0 * TB * ncols);
  k<<<(unsigned)blocks, 256, smem, ctx()->stream>>>(L, ldl, B, ldb, ncols, amax);
  MGB_LAUNCHED("trsm_lu");
  return 0;
}

// amax (may be null, float only): also atomicMax of max |U12| into it; the
// fallback path (other block widths) leaves it alone and returns false in
// *amax_done.
template <typename T>
static int trsm_unit_lower(int tb, int64_t ncols, const T *L, int64_t ldl, T *B,
                           int64_t ldb, unsigned *amax = nullptr,
                           bool *amax_done = nullptr) {
  if (amax_done) *amax_done = amax != nullptr;
  if (ncols <= 0 || tb <= 1) return 0;
  if (tb == kRefBlock) return launch_trsm_warp<T, kRefBlock>(ncols, L, ldl, B, ldb, amax);
  if (tb == kOuterBlock) return launch_trsm_warp<T, kOuterBlock>(ncols, L, ldl, B, ldb, amax);
  if (tb == kOuterBlockLp)
    return launch_trsm_warp<T, kOuterBlockLp>(ncols, L, ldl, B, ldb, amax);
  if (tb == kFusedMaxBw) return launch_trsm_warp<T, kFusedMaxBw>(ncols, L, ldl, B, ldb, amax);
  if (amax_done) *amax_done = false;
  return trsm_left_t<T>(true, false, true, tb, ncols, L, ldl, B, ldb, nullptr);
}

// ---- the mixed look-ahead's operands in one launch --------------------------
// After a fused block (TB pivots, its net row map on the device), the
// split tensor-core update of the next block's nn columns needs those
// columns swapped, U12 = L11^{-1} A12 solved, U12 and L21 packed as FP16
// hi + remainder -- otherwise four launches on the look-ahead's critical
// path.  One launch, two roles:
//  * CTAs [0, ncb): eight columns each, one warp per column: the block's row
//    swaps on the column (laswp_kernel's moves), the solve (the arithmetic of
//    trsm_unit_warp_kernel, with L11 staged by cp.async under the swaps), and
//    the column packed with a power-of-two scale of its own (cinv[j] = its
//    inverse, applied in the product's epilogue);
//  * the other CTAs: L21 (rows ke.., the block's columns) packed with the
//    block's scale s_L from the fused kernel's max, 32-row slabs transposed
//    through shared memory (pack_l21_kernel's output).
// CTA 0 leaves 1/s_L for the epilogue.  A per-column scale keeps every U12
// column's entries as far from FP16's subnormals as the block scale keeps
// the largest.
template <int TB>
__global__ void __launch_bounds__(256)
    la_prep_kernel(float *__restrict__ A, int64_t lda, int64_t n, int64_t kb, int nn,
                   const SwapMap *__restrict__ map, const unsigned *__restrict__ amax_l,
                   int ncb, uint16_t *__restrict__ a16, uint16_t *__restrict__ a16lo,
                   uint16_t *__restrict__ b16, uint16_t *__restrict__ b16lo,
                   float *__restrict__ cinv, float *__restrict__ linv) {
  constexpr int RPL = (TB + 31) / 32;
  constexpr int Kp = (TB + 63) / 64 * 64;  // K of the product, zero-padded
  constexpr int LS = TB + 4;                // staged L11's column stride (16-byte)
  static_assert(TB % 4 == 0, "16-byte rows of L11");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *smf = reinterpret_cast<float *>(smem_raw);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ke = kb + TB;
  const float sL = fp16_scale(__ldg(amax_l));
  if (blockIdx.x == 0 && threadIdx.x == 0) *linv = 1.f / sL;  // a power of two: exact
  if ((int)blockIdx.x < ncb) {
    float *Ls = smf;  // Ls[k*LS + i] = L(i, k)
    int32_t *spos = reinterpret_cast<int32_t *>(smf + TB * LS);
    int32_t *ssrc = spos + 2 * kSwapMax;
    // the warp's column, rows kb..ke, after the swaps
    float *top = reinterpret_cast<float *>(ssrc + 2 * kSwapMax) + warp * TB;
    const float *L = A + kb + kb * lda;
    // L11 staged by asynchronous copies, a warp per column: 16 bytes at a
    // time when the columns start on 16-byte boundaries
    if (lda % 4 == 0 && (reinterpret_cast<uintptr_t>(L) & 15) == 0) {
      for (int k = warp; k < TB; k += 8)
        for (int c = lane; c < TB / 4; c += 32) {
          const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&Ls[k * LS + 4 * c]);
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst),
                       "l"(&L[4 * c + (int64_t)k * lda])
                       : "memory");
        }
    } else {
      for (int k = warp; k < TB; k += 8)
        for (int i = lane; i < TB; i += 32) {
          const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&Ls[k * LS + i]);
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst),
                       "l"(&L[i + (int64_t)k * lda])
                       : "memory");
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    // every map slot at once (the entries past cnt are not used), and the
    // column's top rows before the swaps, in flight together
    for (int r = threadIdx.x; r < 2 * kSwapMax; r += 256) {
      spos[r] = __ldg(&map->pos[r]);
      ssrc[r] = __ldg(&map->src[r]);
    }
    const int cnt = __ldg(&map->cnt);
    const int j = (int)blockIdx.x * 8 + warp;
    float *col = A + (ke + j) * lda;
    float x[RPL];
    if (j < nn) {
#pragma unroll
      for (int r = 0; r < RPL; r++) {
        const int i = lane + 32 * r;
        x[r] = i < TB ? col[kb + i] : 0.f;
      }
    }
    __syncthreads();
    if (j < nn) {
      constexpr int MPL = 2 * kSwapMax / 32;  // map entries per lane
      float v[MPL];
#pragma unroll
      for (int q = 0; q < MPL; q++)
        if (lane + 32 * q < cnt) v[q] = col[ssrc[lane + 32 * q]];
#pragma unroll
      for (int r = 0; r < RPL; r++)
        if (lane + 32 * r < TB) top[lane + 32 * r] = x[r];
      __syncwarp();
      // the moves (laswp_kernel's), the top rows' new values kept on chip
#pragma unroll
      for (int q = 0; q < MPL; q++)
        if (lane + 32 * q < cnt) {
          const int32_t p = spos[lane + 32 * q];
          col[p] = v[q];
          if (p < ke) top[p - kb] = v[q];
        }
      __syncwarp();
#pragma unroll
      for (int r = 0; r < RPL; r++)
        if (lane + 32 * r < TB) x[r] = top[lane + 32 * r];
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    if (j >= nn) return;
    float *b = col + kb;
#pragma unroll
    for (int k = 0; k < TB - 1; k++) {
      const float xk = __shfl_sync(0xffffffffu, x[k / 32], k % 32);
#pragma unroll
      for (int r = k / 32; r < RPL; r++) {
        const int i = lane + 32 * r;
        if (i > k && i < TB) x[r] = fmaf(-Ls[k * LS + i], xk, x[r]);
      }
    }
    float m = 0.f;  // NaN ignored here; it propagates through the product
#pragma unroll
    for (int r = 0; r < RPL; r++) {
      const int i = lane + 32 * r;
      if (i > 0 && i < TB) b[i] = x[r];
      if (i < TB) m = fmaxf(m, fabsf(x[r]));
    }
    for (int off = 16; off; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    const float sc = fp16_scale(__float_as_uint(m));
    if (lane == 0) cinv[j] = 1.f / sc;
    uint16_t *oh = b16 + (int64_t)j * Kp, *ol = b16lo + (int64_t)j * Kp;
#pragma unroll
    for (int r = 0; r < Kp / 32; r++) {
      const int i = lane + 32 * r;
      float vv = 0.f;
#pragma unroll
      for (int q = 0; q < RPL; q++)
        if (q == r && i < TB) vv = sc * x[q];
      const uint16_t h = to16<0>(vv);
      oh[i] = h;
      ol[i] = to16<0>(vv - from16<0>(h));
    }
    return;
  }
  // ---- L21 ----
  const int64_t m = n - ke;
  float *t = smf;  // t[k*33 + r]
  const int64_t nl = (int64_t)gridDim.x - ncb;
  constexpr int nch = Kp / 16;  // 16-entry chunks of an output row
  constexpr int KPW = (TB + 7) / 8;  // columns per warp
  for (int64_t s0 = ((int64_t)blockIdx.x - ncb) * 32; s0 < m; s0 += nl * 32) {
    const int64_t i = s0 + lane;
    // every load of the warp's columns in flight before the first store
    float v[KPW];
    const float *src = A + ke + i + (kb + warp) * lda;
#pragma unroll
    for (int q = 0; q < KPW; q++)
      v[q] = (i < m && warp + 8 * q < TB) ? src[(int64_t)8 * q * lda] : 0.f;
#pragma unroll
    for (int q = 0; q < KPW; q++)
      if (warp + 8 * q < TB) t[(warp + 8 * q) * 33 + lane] = sL * v[q];
    __syncthreads();
    for (int task = threadIdx.x; task < 32 * nch; task += 256) {
      const int r = task & 31, c = task >> 5;
      const int64_t row = s0 + r;
      if (row >= m) continue;
      uint32_t hw[8], lw[8];
#pragma unroll
      for (int e = 0; e < 8; e++) {
        const int k0 = 16 * c + 2 * e;
        const float v0 = k0 < TB ? t[k0 * 33 + r] : 0.f;
        const float v1 = k0 + 1 < TB ? t[(k0 + 1) * 33 + r] : 0.f;
        const uint16_t h0 = to16<0>(v0), h1 = to16<0>(v1);
        const uint16_t l0 = to16<0>(v0 - from16<0>(h0)), l1 = to16<0>(v1 - from16<0>(h1));
        hw[e] = (uint32_t)h0 | ((uint32_t)h1 << 16);
        lw[e] = (uint32_t)l0 | ((uint32_t)l1 << 16);
      }
      uint4 *dh = reinterpret_cast<uint4 *>(a16 + row * Kp + 16 * c);
      uint4 *dl = reinterpret_cast<uint4 *>(a16lo + row * Kp + 16 * c);
      dh[0] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
      dh[1] = make_uint4(hw[4], hw[5], hw[6], hw[7]);
      dl[0] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      dl[1] = make_uint4(lw[4], lw[5], lw[6], lw[7]);
    }
    __syncthreads();
  }
}

// The look-ahead of a fused float block for the split update (lp 2): the
// operands from la_prep_kernel, then C[ke:n, ke:ke+nn] -= L21 U12 on the
// tensor cores with U12's column scales.  The packing buffers are the ones
// lp_trailing_update uses (set 0): the rest of the block's update reuses
// the packed L21 from here.
static int g_la_prep = 1;

// st: the stream the two launches go to (the buffers are looked up, and
// grown if needed, with the library stream current, so that a growth waits
// for that stream's queued users).
static int la_prep_update(int64_t n, float *A, int64_t lda, int64_t kb, int nn,
                          const SwapMap *map, const unsigned *amax_l, cudaStream_t st) {
  constexpr int TB = kFusedMaxBw;
  const int64_t ke = kb + TB, m = n - ke;
  const int Kp = (TB + 63) / 64 * 64;
  const size_t an = (size_t)m * Kp, bn = (size_t)(n - ke) * Kp;
  uint16_t *A16 = (uint16_t *)ws(WS_T0, an * 4);
  uint16_t *B16 = (uint16_t *)ws(WS_T1, bn * 4);
  // (the packing scratch WS_T2 holds the blocks' max slots: a slot of its own)
  float *scb = (float *)ws(WS_LAS, 4096);
  if (!A16 || !B16 || !scb) return MATGB_ERR_NOMEM;
  StreamSwap sw(st);
  float *linv = scb, *cinv = scb + 32;
  auto k = la_prep_kernel<TB>;
  const size_t smem = ((size_t)TB * (TB + 4) + 4 * kSwapMax + 8 * TB) * sizeof(float);
  static bool attr = false;
  if (!attr) {
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  const int ncb = (nn + 7) / 8;
  const int64_t slabs = (m + 31) / 32;
  int64_t nl = 2 * (int64_t)ctx()->sms - ncb;
  if (nl > slabs) nl = slabs;
  if (nl < 1) nl = 1;
  {
    // bytes: the swaps (as laswp's scope counts them), L11, L21 read, both
    // packed operands (hi + remainder) written
    KtScope kt("la_prep", (double)TB * TB * nn,
               4.0 * (4.0 * TB * nn + (double)TB * TB + (double)m * TB) +
                   4.0 * ((double)m + nn) * Kp);
    k<<<(unsigned)(ncb + nl), 256, smem, ctx()->stream>>>(A, lda, n, kb, nn, map, amax_l, ncb,
                                                          A16, A16 + an, B16, B16 + bn, cinv,
                                                          linv);
    MGB_LAUNCHED("la_prep");
  }
  return tc_gemm(0, m, nn, Kp, A16, Kp, B16, Kp, -1.f, linv, 1.f, A + ke + ke * lda, lda, 0,
                 nullptr, A16 + an, B16 + bn, nullptr, cinv);
}

__global__ void iota_kernel(int32_t *p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = (int32_t)i;
}

// X[i, c] = B[perm[i], c]  (pb[i] = b[p[i]] of mat_solve, mat.h:4825-4827)
template <typename T>
__global__ void gather_rows_kernel(int64_t n, int64_t nrhs,
                                   const int32_t *__restrict__ perm,
                                   const T *__restrict__ B, int64_t ldb,
                                   T *__restrict__ X, int64_t ldx) {
  const int64_t tot = n * nrhs;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n, c = e / n;
    X[i + c * ldx] = B[perm[i] + c * ldb];
  }
}

struct PanelPlan {
  int cs, w, rpc;
  size_t smem;
};

template <typename T>
struct PanelState {
  static bool ready;
  static int maxcs;
};
template <typename T>
bool PanelState<T>::ready = false;
template <typename T>
int PanelState<T>::maxcs = 8;

template <typename T>
static int panel_setup() {
  if (PanelState<T>::ready) return 0;
  auto kern = lu_panel_kernel<T>;  // attribute and launch use this pointer
  MGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kSmemMax));
  // 16-CTA clusters are non-portable: use them only if the device accepts one.
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed,
                           1) == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kPanelThreads);
    cfg.dynamicSmemBytes = kSmemMax;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 16;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess &&
        nclusters > 0)
      PanelState<T>::maxcs = 16;
  }
  cudaGetLastError();
  PanelState<T>::ready = true;
  return 0;
}

// Smallest cluster that holds the panel with at most 2 rows per thread;
// the full reference width (24) unless even the largest cluster cannot hold
// it, then the widest divisor of 24 that fits.
template <typename T>
static int plan_panel(int64_t m, int wmax, PanelPlan *pl) {
  static const int widths[] = {24, 12, 8, 6, 4, 3, 2, 1};
  const int maxcs = PanelState<T>::maxcs;
  for (int wi = 0; wi < 8; wi++) {
    int w = widths[wi];
    if (w > wmax) continue;
    for (int cs = 1; cs <= maxcs; cs *= 2) {
      int64_t rpc = (m + cs - 1) / cs;
      size_t sm = panel_smem<T>(cs, w, (int)rpc);
      if (sm > (size_t)kSmemMax) continue;
      if (rpc > 2 * kPanelThreads && cs < maxcs) {
        int64_t rpc2 = (m + 2 * cs - 1) / (2 * cs);
        if (panel_smem<T>(2 * cs, w, (int)rpc2) <= (size_t)kSmemMax) continue;
      }
      pl->cs = cs;
      pl->w = w;
      pl->rpc = (int)rpc;
      pl->smem = sm;
      return 0;
    }
  }
  return set_error(MATGB_ERR_ARG, "LU panel of %lld rows does not fit",
                   (long long)m);
}

template <typename T, int R, int NT>
static int launch_reg_panel(T *A, int64_t lda, int64_t n, int64_t k0, int cs,
                            int rpc, int32_t *ipiv, T eps) {
  auto kern = lu_panel_reg_kernel<T, R, NT>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaGetLastError();
    attr = true;
  }
  const double m = (double)(n - k0);
  KtScope kt("lu_panel", m * kW * kW, 2.0 * m * kW * sizeof(T));
  // always a cluster launch (of one CTA too): the column exchange uses
  // cluster shared-memory addressing
  {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = ctx()->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, A, lda, n, k0, rpc, ipiv, eps);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(MATGB_ERR_CUDA,
                       "lu_panel_reg<R=%d,NT=%d> launch (cluster %d, rows %lld, "
                       "rpc %d): %s", R, NT, cs, (long long)(n - k0), rpc,
                       cudaGetErrorString(e));
    }
  }
  MGB_LAUNCHED("lu_panel");
  return 0;
}

// Register-panel candidates (rows per thread, threads per CTA), cheapest
// first; the register budget per thread (24*R values + the hoisted pivot row)
// decides which fit.
template <typename T>
static int try_reg_panel(T *A, int64_t lda, int64_t n, int64_t k0,
                         int32_t *ipiv, T eps, bool *done) {
  const int64_t m = n - k0;
  const int maxcs = PanelState<T>::maxcs;
  *done = false;
  auto pick = [&](int cap) -> int {
    for (int cs = 1; cs <= maxcs; cs *= 2)
      if ((int64_t)cs * cap >= m) return cs;
    return 0;
  };
  if constexpr (sizeof(T) == 4) {
    int cs;
    if ((cs = pick(512))) {
      *done = true;
      return launch_reg_panel<T, 1, 512>(A, lda, n, k0, cs, (int)((m + cs - 1) / cs), ipiv, eps);
    }
    if ((cs = pick(1024))) {
      *done = true;
      return launch_reg_panel<T, 2, 512>(A, lda, n, k0, cs, (int)((m + cs - 1) / cs), ipiv, eps);
    }
    if ((cs = pick(1024))) {
      *done = true;
      return launch_reg_panel<T, 4, 256>(A, lda, n, k0, cs, (int)((m + cs - 1) / cs), ipiv, eps);
    }
  } else {
    int cs;
    if ((cs = pick(256))) {
      *done = true;
      return launch_reg_panel<T, 1, 256>(A, lda, n, k0, cs, (int)((m + cs - 1) / cs), ipiv, eps);
    }
    if ((cs = pick(512))) {
      *done = true;
      return launch_reg_panel<T, 2, 256>(A, lda, n, k0, cs, (int)((m + cs - 1) / cs), ipiv, eps);
    }
  }
  return 0;
}

// Factor the panel rows [k0,n) x cols [k0, k0+w'), w' <= w chosen to fit:
// the register kernel for full 24-column panels that fit a cluster's
// registers, otherwise the shared-memory kernel.
template <typename T>
int lu_panel_t(T *A, int64_t lda, int64_t n, int64_t k0, int w, int32_t *ipiv,
               T eps, int *w_used) {
  MGB_TRY(panel_setup<T>());
  if (w >= kW) {
    bool done = false;
    MGB_TRY(try_reg_panel<T>(A, lda, n, k0, ipiv, eps, &done));
    if (done) {
      *w_used = kW;
      return 0;
    }
  }
  PanelPlan pl;
  MGB_TRY(plan_panel<T>(n - k0, w, &pl));
  const double m = (double)(n - k0);
  KtScope kt("lu_panel", m * pl.w * pl.w, 2.0 * m * pl.w * sizeof(T));
  auto kern = lu_panel_kernel<T>;
  if (pl.cs == 1) {
    kern<<<1, kPanelThreads, pl.smem, ctx()->stream>>>(A, lda, n, k0, pl.w,
                                                        pl.rpc, ipiv, eps);
  } else {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(pl.cs);
    cfg.blockDim = dim3(kPanelThreads);
    cfg.dynamicSmemBytes = pl.smem;
    cfg.stream = ctx()->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = pl.cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, A, lda, n, k0, pl.w, pl.rpc,
                                       ipiv, eps);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(MATGB_ERR_CUDA,
                       "lu_panel launch (cluster %d, rows %lld, w %d, smem %zu): %s",
                       pl.cs, (long long)(n - k0), pl.w, pl.smem,
                       cudaGetErrorString(e));
    }
  }
  MGB_LAUNCHED("lu_panel");
  *w_used = pl.w;
  return 0;
}

// The fused block factorisation when the block fits one cluster's registers
// (float; rows n-kb <= 16 CTAs x 1024); *done = false otherwise.
template <typename T>
static int try_fused_block(T *A, int64_t lda, int64_t n, int64_t kb, int bw,
                           int32_t *ipiv, T eps, bool *done, unsigned *amax_l,
                           SwapMap *bmap) {
  *done = false;
  if constexpr (sizeof(T) != 4) {
    return 0;
  } else {
    if (bw % kW || bw > kFusedMaxBw) return 0;
    MGB_TRY(panel_setup<T>());
    const int maxcs = PanelState<T>::maxcs;
    const int64_t m = n - kb;
    int cs = 0, R = 0;
    for (int c = 1; c <= maxcs && !cs; c *= 2)
      if ((int64_t)c * 512 >= m) { cs = c; R = 1; }
    for (int c = 1; c <= maxcs && !cs; c *= 2)
      if ((int64_t)c * 1024 >= m) { cs = c; R = 2; }
    if (!cs) return 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
    cfg.blockDim = dim3(512);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = ctx()->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const double mm = (double)m;
    KtScope kt("lu_block_fused", mm * bw * bw, 2.0 * mm * bw * sizeof(T));
    cudaError_t e;
    if (R == 1) {
      auto kern = lu_block_fused_kernel<T, 1, 512>;
      cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      e = cudaLaunchKernelEx(&cfg, kern, A, lda, n, kb, bw, ipiv, eps, amax_l, bmap);
    } else {
      auto kern = lu_block_fused_kernel<T, 2, 512>;
      cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      e = cudaLaunchKernelEx(&cfg, kern, A, lda, n, kb, bw, ipiv, eps, amax_l, bmap);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(MATGB_ERR_CUDA, "lu_block_fused launch (cluster %d, R %d): %s",
                       cs, R, cudaGetErrorString(e));
    }
    MGB_LAUNCHED("lu_block_fused");
    *done = true;
    return 0;
  }
}

// Factor the outer block columns [kb, ke) (rows [kb, n)) with 24-column
// panels: swaps, U12 solve and update restricted to the block's columns.
template <typename T>
static int factor_block(int64_t n, T *A, int64_t lda, int64_t kb, int64_t ke,
                        int32_t *ipiv, T eps) {
  for (int64_t jb = kb; jb < ke;) {
    int wmax = (int)((ke - jb) < kRefBlock ? (ke - jb) : kRefBlock);
    int w = 0;
    MGB_TRY(lu_panel_t<T>(A, lda, n, jb, wmax, ipiv, eps, &w));
    const int64_t je = jb + w;
    MGB_TRY(laswp_t<T>(A, lda, kb, jb, je, ke, ipiv, jb, je, nullptr));
    if (je < ke) {
      MGB_TRY(trsm_unit_lower<T>(w, ke - je, A + jb + jb * lda, lda,
                                 A + jb + je * lda, lda));
      MGB_TRY(gemm_skip_t<T>(false, false, n - je, ke - je, w, T(-1),
                             A + je + jb * lda, lda, A + jb + je * lda, lda,
                             T(1), A + je + je * lda, lda, 0, nullptr));
    }
    jb = je;
  }
  return 0;
}

// Library stream + a high-priority stream for the panel chain, and a ring
// of events ordering them.
struct LookAhead {
  cudaStream_t hi = nullptr;
  cudaEvent_t ev[4] = {};
  bool ready = false;
};
static LookAhead g_la;

static int lookahead_setup() {
  if (g_la.ready) return 0;
  int lo = 0, hi = 0;
  MGB_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
  MGB_CUDA(cudaStreamCreateWithPriority(&g_la.hi, cudaStreamNonBlocking, hi));
  for (auto &e : g_la.ev)
    MGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  g_la.ready = true;
  return 0;
}

// Trailing update C[ke:n, c0:c1] -= L21 * U12[:, c0:c1] for outer block
// [kb, ke): SIMT GEMM in T (lp < 0) or the tensor-core path (lp >= 0, float
// only: L21 packed to 16 bits on the block's first call, U12 per call, see
// mixed.cu).
template <typename T>
static int trailing_update(int64_t n, T *A, int64_t lda, int64_t kb,
                           int64_t ke, int64_t c0, int64_t c1, int lp,
                           bool first, unsigned *amax3 = nullptr,
                           bool l21_ready = false, bool u12_ready = false) {
  if (c1 <= c0 || ke >= n) return 0;
  if (lp < 0)
    return gemm_skip_t<T>(false, false, n - ke, c1 - c0, ke - kb, T(-1),
                          A + ke + kb * lda, lda, A + kb + c0 * lda, lda, T(1),
                          A + ke + c0 * lda, lda, 0, nullptr);
  if (lp == 3) {
    // the plain float LU: the three-part split (about 33 bits of each
    // operand), per-row / per-column scales (tc_sgemm.cu)
    if (sizeof(T) != 4) return set_error(MATGB_ERR_ARG, "tensor-core LU is float");
    return tc_sgemm(false, false, n - ke, c1 - c0, ke - kb, -1.f,
                    (const float *)(A + ke + kb * lda), lda,
                    (const float *)(A + kb + c0 * lda), lda, 1.f,
                    (float *)(A + ke + c0 * lda), lda, 0, false, 3);
  }
  if (sizeof(T) != 4) return set_error(MATGB_ERR_ARG, "tensor-core LU is float");
  return lp_trailing_update(n, (float *)A, lda, kb, ke, c0, c1, lp, first, amax3,
                            l21_ready, u12_ready);
}

// Side streams (lowest priority) and events of a chunked factorisation:
// blk[j] after block j's swap map, done[k] after chunk k's last catch-up.
struct ChunkRes {
  cudaStream_t side[kMaxChunks] = {};
  cudaEvent_t done[kMaxChunks] = {};
  std::vector<cudaEvent_t> blk;
  bool ready = false;
};
static ChunkRes g_chunk;

static int chunk_setup(int nblk) {
  if (!g_chunk.ready) {
    int lo = 0, hi = 0;
    MGB_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    for (int k = 0; k < 9; k++) {
      MGB_CUDA(cudaStreamCreateWithPriority(&g_chunk.side[k], cudaStreamNonBlocking, lo));
      MGB_CUDA(cudaEventCreateWithFlags(&g_chunk.done[k], cudaEventDisableTiming));
    }
    g_chunk.ready = true;
  }
  while ((int)g_chunk.blk.size() < nblk) {
    cudaEvent_t e;
    MGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    g_chunk.blk.push_back(e);
  }
  return 0;
}

template <typename T>
int getrf_t(int64_t n, T *A, int64_t lda, int32_t *ipiv, int32_t *perm, T eps,
            int lp, const ArrivalPlan *arr) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (n <= 0) return 0;
  if (n > INT_MAX / 2) return set_error(MATGB_ERR_ARG, "n too large");
  MGB_TRY(lookahead_setup());
  cudaStream_t main = cx->stream, hi = g_la.hi;
  if (perm) {
    iota_kernel<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096),
                  256, 0, main>>>(perm, n);
    MGB_LAUNCHED("iota");
  }
  // float (plain and mixed): 144-column blocks factored by one fused cluster
  // launch each where they fit
  const bool fused = sizeof(T) == 4;
  const int64_t NB = fused ? kFusedMaxBw : lp >= 0 ? kOuterBlockLp : kOuterBlock;
  // the swaps on the columns left of each block are deferred to one pass at
  // the end when a column below the first block fits in shared memory
  const int nblk = (int)((n + NB - 1) / NB);
  SwapMap *maps = nullptr;
  int32_t *gmap = nullptr;
  if (nblk >= 2 && (n - NB) * (int64_t)sizeof(T) <= 200 * 1024 && n * 4 <= 200 * 1024) {
    maps = (SwapMap *)ws(WS_SWM, (size_t)nblk * sizeof(SwapMap));
    gmap = (int32_t *)ws(WS_SWG, (size_t)nblk * n * sizeof(int32_t));
    if (!maps || !gmap) {
      maps = nullptr;
      gmap = nullptr;
      matgb_clear_error();
    }
  }
  const bool defer = maps != nullptr;
  // tensor-core path: per-block max slots (|L21|, |U12| look-ahead, |U12|
  // rest) after the 64 scale floats of the packing scratch, zeroed once here
  // and filled by the factorisation kernels themselves where they can
  unsigned *amax_all = nullptr;
  if (lp == 0 || lp == 2) {
    float *scb = (float *)ws(WS_T2, 256 + (size_t)12 * (nblk + 1));
    if (!scb) return MATGB_ERR_NOMEM;
    amax_all = reinterpret_cast<unsigned *>(scb + 64);
    MGB_CUDA(cudaMemsetAsync(amax_all, 0, (size_t)12 * (nblk + 1), main));
  }
  // Chunked arrival needs every finished block's swap map kept (the late
  // chunks take the swaps then), the columns left of the blocks unswapped
  // until the end (their L21 rows are used in the order they were factored
  // in), the tensor-core updates (per-stream packing buffers) and chunks
  // aligned to the blocks; otherwise every chunk is waited for first.
  if (arr && (!defer || lp < 0 || lp == 3 || arr->cw % NB != 0 || arr->nchunks < 1 ||
              arr->nchunks > 9)) {
    for (int k = 0; k < arr->nchunks; k++) MGB_CUDA(cudaStreamWaitEvent(main, arr->ev[k], 0));
    arr = nullptr;
  }
  if (arr) {
    MGB_TRY(chunk_setup(nblk));
    MGB_CUDA(cudaStreamWaitEvent(main, arr->ev[0], 0));
    // the side streams' packing buffers, at their largest, before the loop
    const int Kp = (int)((NB + 63) / 64 * 64);
    for (int k = 1; k < arr->nchunks; k++)
      for (int q = 0; q < 2; q++)
        if (!ws(WS_CU0 + 3 * (k - 1) + q, (size_t)(n - NB) * Kp * 4) ||
            !ws(WS_CU0 + 3 * (k - 1) + 2, 256))
          return MATGB_ERR_NOMEM;
  }
  std::vector<char> kept((size_t)nblk, 0);
  int joined = 1;  // chunks 0..joined-1 are in the main stream's updates
  auto columns_in = [&]() -> int64_t {
    if (!arr) return n;
    const int64_t e = (int64_t)joined * arr->cw;
    return e < n ? e : n;
  };
  // Chunk k (k >= 1) catches up on side stream k (low priority): once it has
  // arrived and block j's pivots and swap map exist, block j's row swaps,
  // U12 solve and trailing update are applied to its columns, block after
  // block, while the factorisation goes on.  It joins the main stream's
  // updates just before the look-ahead reaches its first block (the main
  // stream waits there for its last catch-up step).
  auto catch_up = [&](int64_t jb) -> int {
    const int j = (int)(jb / NB);
    const int64_t je = jb + NB;
    for (int k = joined; k < arr->nchunks; k++) {
      const int64_t c0 = (int64_t)k * arr->cw;
      const int64_t c1 = c0 + arr->cw < n ? c0 + arr->cw : n;
      if (je > c0) continue;  // (blocks inside a chunk come after its join)
      cudaStream_t sk = g_chunk.side[k];
      if (jb == 0) MGB_CUDA(cudaStreamWaitEvent(sk, arr->ev[k], 0));
      MGB_CUDA(cudaStreamWaitEvent(sk, g_chunk.blk[j], 0));
      StreamSwap sw(sk);
      if (kept[j])
        MGB_TRY(laswp_map<T>(A, lda, c0, c1, 0, 0, &maps[j], nullptr, NB));
      else
        MGB_TRY(laswp_t<T>(A, lda, c0, c1, 0, 0, ipiv, jb, je, nullptr));
      bool u_dummy = false;
      MGB_TRY(trsm_unit_lower<T>((int)NB, c1 - c0, A + jb + jb * lda, lda,
                                 A + jb + c0 * lda, lda, nullptr, &u_dummy));
      // the packing scales from this stream's own max slots (the block's
      // shared slots would be raised by the other chunks' streams while
      // this one's packing reads them)
      if constexpr (sizeof(T) == 4)
        MGB_TRY(lp_trailing_update(n, (float *)A, lda, jb, je, c0, c1, lp, true, nullptr,
                                   false, false, k));
      else
        return set_error(MATGB_ERR_ARG, "chunked LU is float");
      MGB_CUDA(cudaEventRecord(g_chunk.done[k], sk));
    }
    return 0;
  };
  // main -> hi: everything queued so far (input copies, perm init, slots);
  // ev[3] marks the end of each block's remaining update on main
  MGB_CUDA(cudaEventRecord(g_la.ev[0], main));
  MGB_CUDA(cudaStreamWaitEvent(hi, g_la.ev[0], 0));
  MGB_CUDA(cudaEventRecord(g_la.ev[3], main));
  for (int64_t kb = 0; kb < n; kb += NB) {
    const int64_t nb = (n - kb) < NB ? (n - kb) : NB;
    const int64_t ke = kb + nb;
    unsigned *amax3 = amax_all ? amax_all + 3 * (kb / NB) : nullptr;
    bool l21_ready = false;
    // a fused block also writes its net row map (into the deferred pass's
    // slot, or a ring slot), so the swaps below need no map build
    SwapMap *bmap = nullptr;
    {
      StreamSwap sw(hi);
      bool done = false;
      if (fused && nb == NB) {
        bmap = defer ? &maps[kb / NB] : swap_ring_slot();
        MGB_TRY(try_fused_block<T>(A, lda, n, kb, (int)nb, ipiv, eps, &done,
                                   lp == 2 ? amax3 : nullptr, bmap));
      }
      if (!done) bmap = nullptr;
      l21_ready = done && lp == 2;
      if (!done) MGB_TRY(factor_block<T>(n, A, lda, kb, ke, ipiv, eps));
      kept[kb / NB] = defer && (bmap != nullptr || kb > 0);
    }
    MGB_CUDA(cudaEventRecord(g_la.ev[1], hi));
    MGB_CUDA(cudaStreamWaitEvent(main, g_la.ev[1], 0));

    const int64_t nn = (n - ke) < NB ? (n - ke) : NB;
    // the one-launch look-ahead (swaps, U12 solve, both operands packed) of
    // the split update runs on the panel stream, right behind the block
    const bool prep = ke < n && sizeof(T) == 4 && g_la_prep && bmap && lp == 2 && amax3 &&
                      l21_ready && nb == kFusedMaxBw;
    // the look-ahead's columns must have joined (a plan that is too late
    // for them costs a wait here, never a wrong result); the look-ahead
    // then packs this block's L21 afresh
    while (arr && joined < arr->nchunks && columns_in() < ke + nn) {
      MGB_CUDA(cudaStreamWaitEvent(main, arr->ev[joined], 0));
      MGB_CUDA(cudaStreamWaitEvent(main, g_chunk.done[joined], 0));
      if (prep) {
        MGB_CUDA(cudaStreamWaitEvent(hi, arr->ev[joined], 0));
        MGB_CUDA(cudaStreamWaitEvent(hi, g_chunk.done[joined], 0));
      }
      joined++;
    }
    if (prep) {
      // the previous block's remaining update covered these columns (and
      // read the packing buffers this launch rewrites): wait for it, then
      // the look-ahead on the panel stream, no stream hop before the next
      // block.  Main waits for it before its own swaps: run beside them,
      // the look-ahead's launches lose their SMs to the swaps' CTAs.
      MGB_CUDA(cudaStreamWaitEvent(hi, g_la.ev[3], 0));
      MGB_TRY(la_prep_update(n, (float *)A, lda, kb, (int)nn, bmap, amax3, hi));
      MGB_CUDA(cudaEventRecord(g_la.ev[2], hi));
      MGB_CUDA(cudaStreamWaitEvent(main, g_la.ev[2], 0));
    } else if (ke < n) {
      // look-ahead: the next block's columns are swapped, solved and updated
      // first, then the panel stream is released; everything else (the other
      // columns, the columns left of the block, the permutation) follows
      // off the critical path
      if (bmap)
        MGB_TRY(laswp_map<T>(A, lda, ke, ke + nn, 0, 0, bmap, nullptr, nb));
      else
        MGB_TRY(laswp_t<T>(A, lda, ke, ke + nn, 0, 0, ipiv, kb, ke, nullptr));
      bool u12_ready = false;
      MGB_TRY(trsm_unit_lower<T>((int)nb, nn, A + kb + kb * lda, lda,
                                 A + kb + ke * lda, lda, amax3 ? amax3 + 1 : nullptr,
                                 &u12_ready));
      MGB_TRY(trailing_update<T>(n, A, lda, kb, ke, ke, ke + nn, lp, true, amax3,
                                 l21_ready, u12_ready));
      MGB_CUDA(cudaEventRecord(g_la.ev[2], main));
      MGB_CUDA(cudaStreamWaitEvent(hi, g_la.ev[2], 0));
    }
    const int64_t cend = columns_in();
    // the columns right of the look-ahead (and, unless deferred, the columns
    // left of the block) and the permutation; a deferred pass keeps this
    // block's net map
    const int64_t r1 = cend > ke + nn ? cend : ke + nn;
    if (bmap)
      MGB_TRY(laswp_map<T>(A, lda, 0, defer ? 0 : kb, ke + nn, r1, bmap, perm, nb));
    else
      MGB_TRY(laswp_t<T>(A, lda, 0, defer ? 0 : kb, ke + nn, r1, ipiv, kb, ke, perm,
                         defer && kb > 0 ? &maps[kb / NB] : nullptr));
    if (arr && joined < arr->nchunks && nb == NB) {
      // this block's pivots and swap map exist from here on (main stream)
      MGB_CUDA(cudaEventRecord(g_chunk.blk[kb / NB], main));
      MGB_TRY(catch_up(kb));
    }
    if (ke + nn < r1) {
      bool u12_ready = false;
      MGB_TRY(trsm_unit_lower<T>((int)nb, r1 - ke - nn, A + kb + kb * lda, lda,
                                 A + kb + (ke + nn) * lda, lda,
                                 amax3 ? amax3 + 2 : nullptr, &u12_ready));
      MGB_TRY(trailing_update<T>(n, A, lda, kb, ke, ke + nn, r1, lp, false, amax3,
                                 l21_ready, u12_ready));
    }
    MGB_CUDA(cudaEventRecord(g_la.ev[3], main));
  }
  if (defer) MGB_TRY(apply_deferred_swaps<T>(A, lda, n, NB, nblk, maps, gmap));
  return 0;
}

template <typename T>
int getrs_t(int64_t n, int64_t nrhs, const T *LU, int64_t lda,
            const int32_t *perm, const T *B, int64_t ldb, T *X, int64_t ldx) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (n <= 0 || nrhs <= 0) return 0;
  int64_t tot = n * nrhs;
  int64_t blocks = (tot + 255) / 256;
  if (blocks > (int64_t)cx->sms * 16) blocks = (int64_t)cx->sms * 16;
  gather_rows_kernel<T><<<(unsigned)blocks, 256, 0, cx->stream>>>(n, nrhs, perm,
                                                                  B, ldb, X, ldx);
  MGB_LAUNCHED("gather_rows");
  MGB_TRY(trsm_left_t<T>(true, false, true, n, nrhs, LU, lda, X, ldx, nullptr));
  MGB_TRY(trsm_left_t<T>(false, false, false, n, nrhs, LU, lda, X, ldx, nullptr));
  return 0;
}

int precond_solve(bool spd, int64_t n, const float *W, const int32_t *perm,
                  const float *in, float *out) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (n <= 0) return 0;
  if (spd) {
    MGB_CUDA(cudaMemcpyAsync(out, in, (size_t)n * sizeof(float),
                             cudaMemcpyDeviceToDevice, cx->stream));
    MGB_TRY(trsv_t<float>(true, false, false, n, W, n, out, true));
    return trsv_t<float>(true, true, false, n, W, n, out, true);
  }
  int64_t blocks = (n + 255) / 256;
  if (blocks > (int64_t)cx->sms * 16) blocks = (int64_t)cx->sms * 16;
  gather_rows_kernel<float><<<(unsigned)blocks, 256, 0, cx->stream>>>(
      n, 1, perm, in, n, out, n);
  MGB_LAUNCHED("gather_rows");
  MGB_TRY(trsv_t<float>(true, false, true, n, W, n, out, true));
  return trsv_t<float>(false, false, false, n, W, n, out, true);
}

#define MGB_LU_INST(T)                                                         \
  template int laswp_t<T>(T *, int64_t, int64_t, int64_t, int64_t, int64_t,    \
                          const int32_t *, int64_t, int64_t, int32_t *,        \
                          SwapMap *);                                          \
  template int lu_panel_t<T>(T *, int64_t, int64_t, int64_t, int, int32_t *,  \
                             T, int *);                                        \
  template int getrf_t<T>(int64_t, T *, int64_t, int32_t *, int32_t *, T, int,      \
                          const ArrivalPlan *);                                     \
  template int getrs_t<T>(int64_t, int64_t, const T *, int64_t,               \
                          const int32_t *, const T *, int64_t, T *, int64_t);
MGB_LU_INST(float)
MGB_LU_INST(double)
#undef MGB_LU_INST

// Whether a panel exchange gave up waiting since the last clear (call after
// the stream has been synchronised).
int lu_wait_error(int clear) {
  int h = 0;
  MGB_CUDA(cudaMemcpyFromSymbol(&h, g_lu_wait_err, sizeof(int)));
  if (clear && h) {
    const int z = 0;
    MGB_CUDA(cudaMemcpyToSymbol(g_lu_wait_err, &z, sizeof(int)));
  }
  return h;
}

int laswp(elem_t *A, int64_t lda, int64_t c0, int64_t c1, int64_t c2,
          int64_t c3, const int32_t *ipiv, int64_t k1, int64_t k2) {
  return laswp_t<elem_t>(A, lda, c0, c1, c2, c3, ipiv, k1, k2, nullptr);
}

// The plain LU (mat_plu, mat_solve, matgb_getrf_dev): the pivot sequence
// must follow the reference's on every data-determined step.  The
// three-product FP16 split (about 22 bits per operand) is noisier than FP32
// -- on the 8192 N(0,1) plain config it changed a pivot at step 6370, where
// FP32 updates follow the reference up to step 8116, the first step at which
// the reference's own float and double pivots part.  The float build's
// orders from 1024 up therefore take the six-product three-part split (about
// 33 bits per operand, more accurate than the FP32 products it replaces)
// unless matgb_plain_tensor_core(0) chose the SIMT GEMM.
int getrf(int64_t n, elem_t *A, int64_t lda, int32_t *ipiv, int32_t *perm) {
  const int lp = (sizeof(elem_t) == 4 && plain_tc_on() && n >= kPlainTcMinN) ? 3 : -1;
  return getrf_t<elem_t>(n, A, lda, ipiv, perm, kPivotEps, lp);
}

int getrs(int64_t n, int64_t nrhs, const elem_t *LU, int64_t lda,
          const int32_t *perm, const elem_t *B, int64_t ldb, elem_t *X,
          int64_t ldx) {
  return getrs_t<elem_t>(n, nrhs, LU, lda, perm, B, ldb, X, ldx);
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_getrf_dev(size_t n, mat_elem_t *A, size_t lda, int32_t *ipiv,
                    int32_t *perm) {
  if (lda < n) return set_error(MATGB_ERR_ARG, "getrf: lda < n");
  if (n > 0 && !ipiv) return set_error(MATGB_ERR_ARG, "getrf: ipiv is NULL");
  return getrf((int64_t)n, A, (int64_t)lda, ipiv, perm);
}

int matgb_getrs_dev(size_t n, size_t nrhs, const mat_elem_t *LU, size_t lda,
                    const int32_t *perm, const mat_elem_t *B, size_t ldb,
                    mat_elem_t *X, size_t ldx) {
  if (lda < n || ldb < n || ldx < n)
    return set_error(MATGB_ERR_ARG, "getrs: leading dimension too small");
  if (B == X) return set_error(MATGB_ERR_ARG, "getrs: B and X must differ");
  return getrs((int64_t)n, (int64_t)nrhs, LU, (int64_t)lda, perm, B,
               (int64_t)ldb, X, (int64_t)ldx);
}

int matgb_la_prep(int on) {
  const int prev = g_la_prep;
  if (on >= 0) g_la_prep = on ? 1 : 0;
  return prev;
}

}  // extern "C"
