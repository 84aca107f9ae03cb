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
//  * Outer blocks of 96 columns: after each inner panel the swaps go to the
//    rest of the outer block, then a TRSM and a skinny GEMM; after each outer
//    block the swaps go to all other columns (and to the permutation vector),
//    then TRSM for U12 and the big GEMM (K = 96) for the trailing matrix.
#include <cooperative_groups.h>
#include <limits.h>

#include "internal.cuh"

namespace cg = cooperative_groups;

namespace mgb {

constexpr int kPanelThreads = 512;
constexpr int kPanelWarps = kPanelThreads / 32;
constexpr int kRefBlock = 24;  // MAT_PLU_BLOCK_SIZE, mat.h:4196
constexpr int kOuterBlock = 96;
constexpr int kSmemMax = 227 * 1024;

__device__ __forceinline__ elem_t piv_key(elem_t v, bool first) {
  // Reproduces mat__amax_scalar + mat__iamax on NaNs: a NaN at the first
  // position wins (max becomes NaN, no index compares equal, index 0 is
  // returned); NaNs elsewhere never win.
  elem_t a = fabs(v);
  if (a != a) return first ? (elem_t)INFINITY : (elem_t)-1;
  return a;
}

__device__ __forceinline__ bool better(elem_t k1, int i1, elem_t k2, int i2) {
  return k1 > k2 || (k1 == k2 && i1 < i2);
}

static size_t panel_smem(int cs, int w, int rpc) {
  size_t t = (size_t)w * rpc + kPanelWarps + 2 * cs + 2 * (size_t)cs * w +
             2 * (size_t)w;
  return t * sizeof(elem_t) + (kPanelWarps + 2 * cs) * sizeof(int);
}

// Factor rows [k0, n) x columns [k0, k0+w) of A in place.  ipiv[k0+kk] gets
// the global row swapped into row k0+kk.  One cluster; CTA c holds panel rows
// [c*rpc, (c+1)*rpc).  Thread tid owns local rows tid, tid+512, ...
__global__ void __launch_bounds__(kPanelThreads, 1)
    lu_panel_kernel(elem_t *__restrict__ A, int64_t lda, int64_t n, int64_t k0,
                    int w, int rpc, int32_t *__restrict__ ipiv) {
  cg::cluster_group cluster = cg::this_cluster();
  const int CS = (int)cluster.num_blocks();
  const int c = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t m = n - k0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  elem_t *P = (elem_t *)smem_raw;
  elem_t *wkey = P + (size_t)w * rpc;
  elem_t *xkey = wkey + kPanelWarps;
  elem_t *xval = xkey + 2 * CS;
  elem_t *kval = xval + 2 * (size_t)CS * w;
  int *widx = (int *)(kval + 2 * w);
  int *xidx = widx + kPanelWarps;

  const int64_t rbase = (int64_t)c * rpc;
  for (int r = tid; r < rpc; r += kPanelThreads) {
    const int64_t pr = rbase + r;
    for (int j = 0; j < w; j++)
      P[(size_t)j * rpc + r] = pr < m ? A[(k0 + pr) + (k0 + j) * lda] : elem_t(0);
  }

  for (int kk = 0; kk < w; kk++) {
    const int buf = kk & 1;
    // 1. arg-max of |P[kk][r]| over my rows with panel row >= kk
    elem_t bk = (elem_t)-2;
    int bi = INT_MAX;
    for (int r = tid; r < rpc; r += kPanelThreads) {
      const int64_t pr = rbase + r;
      if (pr >= kk && pr < m) {
        elem_t key = piv_key(P[(size_t)kk * rpc + r], pr == kk);
        if (better(key, (int)pr, bk, bi)) {
          bk = key;
          bi = (int)pr;
        }
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      elem_t ok = __shfl_down_sync(0xffffffffu, bk, off);
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
    elem_t ck = wkey[0];
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
        elem_t v = (ci != INT_MAX) ? P[(size_t)j * rpc + (ci - rbase)] : elem_t(0);
        elem_t *dst = cluster.map_shared_rank(xval, q);
        dst[((size_t)buf * CS + c) * w + j] = v;
      } else if (t < nval + CS) {
        const int q = t - nval;
        elem_t *dk = cluster.map_shared_rank(xkey, q);
        int *di = cluster.map_shared_rank(xidx, q);
        dk[buf * CS + c] = ck;
        di[buf * CS + c] = ci;
      } else {
        const int u = t - nval - CS;
        const int q = u / w, j = u % w;
        elem_t *dst = cluster.map_shared_rank(kval, q);
        dst[(size_t)buf * w + j] = P[(size_t)j * rpc + (kk - rbase)];
      }
    }
    cluster.sync();
    // 3. winner over the cluster (every thread, same answer)
    int wc = 0;
    elem_t gk = xkey[buf * CS];
    int gi = xidx[buf * CS];
    for (int q = 1; q < CS; q++)
      if (better(xkey[buf * CS + q], xidx[buf * CS + q], gk, gi)) {
        gk = xkey[buf * CS + q];
        gi = xidx[buf * CS + q];
        wc = q;
      }
    const elem_t *u = xval + ((size_t)buf * CS + wc) * w;
    const elem_t *kv = kval + (size_t)buf * w;
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
    const elem_t piv = u[kk];
    if (!(fabs(piv) < kPivotEps)) {
      const elem_t inv = elem_t(1) / piv;
      for (int r = tid; r < rpc; r += kPanelThreads) {
        const int64_t pr = rbase + r;
        if (pr > kk && pr < m) {
          const elem_t l = P[(size_t)kk * rpc + r] * inv;
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

// Apply the swaps ipiv[k1..k2) (global row indices) in order to columns
// [c0,c1) and [c2,c3), and, if perm is given, to the permutation vector.
__global__ void laswp_kernel(elem_t *__restrict__ A, int64_t lda, int64_t c0,
                             int64_t c1, int64_t c2, int64_t c3,
                             const int32_t *__restrict__ ipiv, int64_t k1,
                             int64_t k2, int32_t *__restrict__ perm) {
  __shared__ int32_t sp[kOuterBlock];
  const int nk = (int)(k2 - k1);
  for (int i = threadIdx.x; i < nk; i += blockDim.x) sp[i] = ipiv[k1 + i];
  __syncthreads();
  const int64_t na = c1 - c0, nb = c3 - c2;
  const int64_t total = na + nb + (perm ? 1 : 0);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (t < na + nb) {
      const int64_t col = t < na ? c0 + t : c2 + (t - na);
      elem_t *a = A + col * lda;
      for (int i = 0; i < nk; i++) {
        const int64_t k = k1 + i, p = sp[i];
        if (p != k) {
          elem_t x = a[k];
          a[k] = a[p];
          a[p] = x;
        }
      }
    } else {
      for (int i = 0; i < nk; i++) {
        const int64_t k = k1 + i, p = sp[i];
        if (p != k) {
          int32_t x = perm[k];
          perm[k] = perm[p];
          perm[p] = x;
        }
      }
    }
  }
}

__global__ void iota_kernel(int32_t *p, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = (int32_t)i;
}

// X[i, c] = B[perm[i], c]  (pb[i] = b[p[i]] of mat_solve, mat.h:4825-4827)
__global__ void gather_rows_kernel(int64_t n, int64_t nrhs,
                                   const int32_t *__restrict__ perm,
                                   const elem_t *__restrict__ B, int64_t ldb,
                                   elem_t *__restrict__ X, int64_t ldx) {
  const int64_t tot = n * nrhs;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % n, c = e / n;
    X[i + c * ldx] = B[perm[i] + c * ldb];
  }
}

static int laswp_perm(elem_t *A, int64_t lda, int64_t c0, int64_t c1,
                      int64_t c2, int64_t c3, const int32_t *ipiv, int64_t k1,
                      int64_t k2, int32_t *perm) {
  const int64_t total = (c1 - c0) + (c3 - c2) + (perm ? 1 : 0);
  if (total <= 0 || k2 <= k1) return 0;
  const int threads = 128;
  int64_t blocks = (total + threads - 1) / threads;
  KtScope kt("laswp", 0.0, 4.0 * (k2 - k1) * total * sizeof(elem_t));
  laswp_kernel<<<(unsigned)blocks, threads, 0, ctx()->stream>>>(
      A, lda, c0, c1, c2, c3, ipiv, k1, k2, perm);
  MGB_LAUNCHED("laswp");
  return 0;
}

int laswp(elem_t *A, int64_t lda, int64_t c0, int64_t c1, int64_t c2,
          int64_t c3, const int32_t *ipiv, int64_t k1, int64_t k2) {
  return laswp_perm(A, lda, c0, c1, c2, c3, ipiv, k1, k2, nullptr);
}

struct PanelPlan {
  int cs, w, rpc;
  size_t smem;
};

static bool g_panel_ready = false;
static int g_panel_maxcs = 8;

static int panel_setup() {
  if (g_panel_ready) return 0;
  MGB_CUDA(cudaFuncSetAttribute(lu_panel_kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kSmemMax));
  // 16-CTA clusters are non-portable: use them only if the device accepts one.
  if (cudaFuncSetAttribute(lu_panel_kernel,
                           cudaFuncAttributeNonPortableClusterSizeAllowed,
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
    if (cudaOccupancyMaxActiveClusters(&nclusters, lu_panel_kernel, &cfg) ==
            cudaSuccess &&
        nclusters > 0)
      g_panel_maxcs = 16;
  }
  cudaGetLastError();
  g_panel_ready = true;
  return 0;
}

// Smallest cluster that holds the panel with at most 2 rows per thread;
// the full reference width (24) unless even the largest cluster cannot hold
// it, then the widest divisor of 24 that fits.
static int plan_panel(int64_t m, int wmax, PanelPlan *pl) {
  static const int widths[] = {24, 12, 8, 6, 4, 3, 2, 1};
  for (int wi = 0; wi < 8; wi++) {
    int w = widths[wi];
    if (w > wmax) continue;
    for (int cs = 1; cs <= g_panel_maxcs; cs *= 2) {
      int64_t rpc = (m + cs - 1) / cs;
      size_t sm = panel_smem(cs, w, (int)rpc);
      if (sm > (size_t)kSmemMax) continue;
      if (rpc > 2 * kPanelThreads && cs < g_panel_maxcs) {
        // prefer more CTAs while that still fits
        int64_t rpc2 = (m + 2 * cs - 1) / (2 * cs);
        if (panel_smem(2 * cs, w, (int)rpc2) <= (size_t)kSmemMax) continue;
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

static int launch_panel(elem_t *A, int64_t lda, int64_t n, int64_t k0,
                        const PanelPlan &pl, int32_t *ipiv) {
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
  const double m = (double)(n - k0);
  KtScope kt("lu_panel", m * pl.w * pl.w, 2.0 * m * pl.w * sizeof(elem_t));
  MGB_CUDA(cudaLaunchKernelEx(&cfg, lu_panel_kernel, A, lda, n, k0, pl.w,
                              pl.rpc, ipiv));
  MGB_LAUNCHED("lu_panel");
  return 0;
}

int getrf(int64_t n, elem_t *A, int64_t lda, int32_t *ipiv, int32_t *perm) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (n <= 0) return 0;
  if (n > INT_MAX / 2) return set_error(MATGB_ERR_ARG, "n too large");
  MGB_TRY(panel_setup());
  if (perm) {
    iota_kernel<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096),
                  256, 0, cx->stream>>>(perm, n);
    MGB_LAUNCHED("iota");
  }
  for (int64_t kb = 0; kb < n; kb += kOuterBlock) {
    const int64_t nb = (n - kb) < kOuterBlock ? (n - kb) : kOuterBlock;
    const int64_t ke = kb + nb;
    for (int64_t jb = kb; jb < ke;) {
      PanelPlan pl;
      int wmax = (int)((ke - jb) < kRefBlock ? (ke - jb) : kRefBlock);
      MGB_TRY(plan_panel(n - jb, wmax, &pl));
      if (pl.w > wmax) pl.w = wmax;
      const int64_t je = jb + pl.w;
      MGB_TRY(launch_panel(A, lda, n, jb, pl, ipiv));
      MGB_TRY(laswp_perm(A, lda, kb, jb, je, ke, ipiv, jb, je, nullptr));
      if (je < ke) {
        MGB_TRY(trsm_left(true, false, true, pl.w, ke - je, A + jb + jb * lda,
                          lda, A + jb + je * lda, lda, nullptr));
        MGB_TRY(gemm(false, false, n - je, ke - je, pl.w, elem_t(-1),
                     A + je + jb * lda, lda, A + jb + je * lda, lda, elem_t(1),
                     A + je + je * lda, lda, 0));
      }
      jb = je;
    }
    MGB_TRY(laswp_perm(A, lda, 0, kb, ke, n, ipiv, kb, ke, perm));
    if (ke < n) {
      MGB_TRY(trsm_left(true, false, true, nb, n - ke, A + kb + kb * lda, lda,
                        A + kb + ke * lda, lda, nullptr));
      MGB_TRY(gemm(false, false, n - ke, n - ke, nb, elem_t(-1),
                   A + ke + kb * lda, lda, A + kb + ke * lda, lda, elem_t(1),
                   A + ke + ke * lda, lda, 0));
    }
  }
  return 0;
}

int getrs(int64_t n, int64_t nrhs, const elem_t *LU, int64_t lda,
          const int32_t *perm, const elem_t *B, int64_t ldb, elem_t *X,
          int64_t ldx) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (n <= 0 || nrhs <= 0) return 0;
  int64_t tot = n * nrhs;
  int64_t blocks = (tot + 255) / 256;
  if (blocks > (int64_t)cx->sms * 16) blocks = (int64_t)cx->sms * 16;
  gather_rows_kernel<<<(unsigned)blocks, 256, 0, cx->stream>>>(n, nrhs, perm, B,
                                                               ldb, X, ldx);
  MGB_LAUNCHED("gather_rows");
  MGB_TRY(trsm_left(true, false, true, n, nrhs, LU, lda, X, ldx, nullptr));
  MGB_TRY(trsm_left(false, false, false, n, nrhs, LU, lda, X, ldx, nullptr));
  return 0;
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

}  // extern "C"
