// Full-pivoting LU (mat_lu, mat.h:4476-4574), bit-identical to the
// reference's scalar elimination.
//
// Each step k of the reference:
//   - scans the trailing block (rows then columns from (k, k)) for the
//     first entry whose magnitude is strictly larger than |a_kk|;
//   - skips the step when that magnitude is below MAT_DEFAULT_EPSILON;
//   - swaps whole rows k <-> pr, then whole columns k <-> pc;
//   - divides the column below the pivot by the pivot through
//     inv = 1 / a_kk (l = a_ik * inv);
//   - subtracts l * a_kj from every trailing entry, the product rounded
//     before the subtraction.
// Every step needs the whole updated trailing block for its pivot search,
// so the work is a chain of rank-1 updates; there is nothing to block.  It
// is bound by the memory traffic of the trailing block (read and written
// once per step) and by the chain's per-step latency.
//
// GPU form: one launch per step, over the trailing block in 64 x 32 tiles.
// Launch k applies step k's update (the multipliers and pivot row were left
// in place by launch k-1) and, over the values it has just written, finds
// each CTA's best candidate for step k+1.  The last CTA to finish (a ticket
// counter) reduces those candidates, records step k+1's pivot and performs
// its row swap, column swap and column scaling, so that launch k+1 again
// finds its operands in place.  Launch -1 only searches.
//
// Pivot order: the reference keeps the FIRST entry, in row-major order from
// (k, k), of the largest magnitude; NaN entries never win a comparison, and
// a NaN at (k, k) keeps the pivot there.  Candidates are therefore compared
// on (|a|, then the smaller row-major index i*n + j); NaN counts as -1.
#include <algorithm>

#include "internal.cuh"

namespace mgb {
namespace {

constexpr int kFullRows = 64;      // tile rows (one per thread)
constexpr int kFullTileCols = 32;  // tile columns
constexpr int kFullThreads = 256;  // 64 rows x 4 column groups
constexpr int kFullGroups = kFullThreads / kFullRows;      // column groups
constexpr int kFullCols = kFullTileCols / kFullGroups;     // columns per thread
constexpr int kFullBatch = 4;      // swap entries per thread in flight

// Candidate: magnitude (-1 for NaN / none) and row-major index.
template <typename T>
struct Cand {
  T v;
  unsigned long long r;
};

template <typename T>
__device__ __forceinline__ bool cand_better(T v1, unsigned long long r1, T v2,
                                            unsigned long long r2) {
  return v1 > v2 || (v1 == v2 && r1 < r2);
}

template <typename T>
__device__ __forceinline__ T mag_or_neg(T a) {
  return isnan(a) ? T(-1) : fabs(a);
}

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Block-wide best candidate, returned to every thread.
template <typename T>
__device__ Cand<T> block_best(T v, unsigned long long r, Cand<T> *sm) {
  for (int o = 16; o > 0; o >>= 1) {
    const T v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const unsigned long long r2 = __shfl_xor_sync(0xffffffffu, r, o);
    if (cand_better(v2, r2, v, r)) {
      v = v2;
      r = r2;
    }
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) sm[w] = Cand<T>{v, r};
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kFullThreads / 32; i++)
      if (cand_better(sm[i].v, sm[i].r, v, r)) {
        v = sm[i].v;
        r = sm[i].r;
      }
    sm[0] = Cand<T>{v, r};
  }
  __syncthreads();
  return sm[0];
}

__global__ void full_iota_kernel(int32_t *__restrict__ p, int32_t *__restrict__ q,
                                 int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = q[i] = (int32_t)i;
}

// Scratch of one factorisation (device).
struct FullPivState {
  unsigned ticket;
  unsigned pad[3];
};

// Launch for step k (k = -1: search only).  m = n - k - 1 is the order of
// the trailing block T that this launch updates and then searches.
template <typename T>
__global__ void __launch_bounds__(kFullThreads, 3)
    lu_full_step_kernel(T *__restrict__ A, int64_t n, int64_t lda, int64_t k,
                        FullPivState *st, T *part_v,
                        unsigned long long *part_r, int32_t *rowpiv,
                        int32_t *colpiv, int32_t *skip, T eps) {
  __shared__ Cand<T> sm[kFullThreads / 32];
  __shared__ unsigned s_last;
  // Launched as a programmatic dependent of the previous step: wait for it
  // to complete (its writes visible), then let the next step's CTAs be
  // scheduled; they wait in turn, on slots this grid no longer needs.
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;");
  const int64_t b = k + 1;  // first row and column of T
  const int64_t m = n - b;
  const bool update = k >= 0 && skip[k] == 0;
  const bool search = b + 1 < n;  // step b exists (steps run to n - 2)
  const int64_t ntr = (m + kFullRows - 1) / kFullRows;
  const int64_t ntc = (m + kFullTileCols - 1) / kFullTileCols;
  const int ti = threadIdx.x % kFullRows, tg = threadIdx.x / kFullRows;

  T bv = T(-1);
  unsigned long long br = ~0ull;
  for (int64_t t = blockIdx.x; t < ntr * ntc; t += gridDim.x) {
    const int64_t i = b + (t % ntr) * kFullRows + ti;
    const int64_t j0 = b + (t / ntr) * kFullTileCols + tg;
    if (i >= n || j0 >= n) continue;
    // columns j0, j0 + 4, ... below n
    const int64_t left = (n - j0 + kFullGroups - 1) / kFullGroups;
    const int nq = left < kFullCols ? (int)left : kFullCols;
    const int64_t step = kFullGroups * lda;
    T *pa = A + i + j0 * lda;
    const T *pu = A + k + j0 * lda;
    T a[kFullCols], u[kFullCols];
    const T l = update ? pa[(k - j0) * lda] : T(0);
#pragma unroll
    for (int q = 0; q < kFullCols; q++)
      if (q < nq) {
        a[q] = pa[q * step];
        u[q] = update ? pu[q * step] : T(0);
      }
    const unsigned long long r0 = (unsigned long long)i * n + j0;
#pragma unroll
    for (int q = 0; q < kFullCols; q++)
      if (q < nq) {
        if (update) {
          a[q] = sub_rn(a[q], mul_rn(l, u[q]));
          pa[q * step] = a[q];
        }
        const T v = mag_or_neg(a[q]);
        if (cand_better(v, r0 + q * kFullGroups, bv, br)) {
          bv = v;
          br = r0 + q * kFullGroups;
        }
      }
  }
  if (!search) return;

  // The barriers in block_best order every thread's updated entries before
  // thread 0's device-wide fence and ticket, so the last CTA reads them.
  const Cand<T> best = block_best(bv, br, sm);
  if (threadIdx.x == 0) {
    part_v[blockIdx.x] = best.v;
    part_r[blockIdx.x] = best.r;
    __threadfence();
    s_last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();

  // Last CTA: step b's pivot over all CTAs' candidates.
  bv = T(-1);
  br = ~0ull;
  for (int c = threadIdx.x; c < (int)gridDim.x; c += kFullThreads) {
    const T v = __ldcg(part_v + c);
    const unsigned long long r = __ldcg(part_r + c);
    if (cand_better(v, r, bv, br)) {
      bv = v;
      br = r;
    }
  }
  const Cand<T> all = block_best(bv, br, sm);
  const T akk = __ldcg(A + b + b * lda);
  int64_t pr = b, pc = b;
  T mx = fabs(akk);
  if (!isnan(akk) && all.v > mx) {
    pr = (int64_t)(all.r / (unsigned long long)n);
    pc = (int64_t)(all.r % (unsigned long long)n);
    mx = all.v;
  }
  const bool skp = mx < eps;  // false for NaN
  if (skp) pr = pc = b;
  if (threadIdx.x == 0) {
    rowpiv[b] = (int32_t)pr;
    colpiv[b] = (int32_t)pc;
    skip[b] = skp ? 1 : 0;
    st->ticket = 0;
  }
  if (skp) return;

  // Step b's swaps and scaling in one pass.  Each changed entry becomes
  // new(i, j) = old(s(i), t(j)) with s = (b pr), t = (b pc), and the column
  // below the pivot is then multiplied by inv = 1 / new(b, b).  The four
  // entries of rows {b, pr} x columns {b, pc} are read by every thread
  // before any store; every other changed entry is read and written by the
  // same thread, so no other ordering is needed.
  const T o_bb = __ldcg(A + b + b * lda), o_bc = __ldcg(A + b + pc * lda);
  const T o_rb = __ldcg(A + pr + b * lda), o_rc = __ldcg(A + pr + pc * lda);
  __syncthreads();
  const T inv = T(1) / o_rc;
  if (threadIdx.x == 0) {
    A[b + b * lda] = o_rc;
    if (pc != b) A[b + pc * lda] = o_rb;
    if (pr != b) A[pr + b * lda] = mul_rn(o_bc, inv);  // pr > b: scaled
    if (pr != b && pc != b) A[pr + pc * lda] = o_bb;
  }
  for (int64_t base = threadIdx.x; base < n;
       base += (int64_t)kFullBatch * kFullThreads) {
    T x[kFullBatch], y[kFullBatch], cb[kFullBatch], cp[kFullBatch];
    bool rw[kFullBatch], cl[kFullBatch];
#pragma unroll
    for (int u = 0; u < kFullBatch; u++) {
      const int64_t j = base + (int64_t)u * kFullThreads;  // also a row i
      // rows b and pr, columns other than b and pc
      rw[u] = pr != b && j < n && j != b && j != pc;
      // columns b and pc, rows other than b and pr: swap (pc != b) and
      // scale (rows below b)
      cl[u] = j < n && j != b && j != pr && (pc != b || j > b);
      if (rw[u]) {
        x[u] = __ldcg(A + b + j * lda);
        y[u] = __ldcg(A + pr + j * lda);
      }
      if (cl[u]) {
        cb[u] = __ldcg(A + j + b * lda);
        cp[u] = pc != b ? __ldcg(A + j + pc * lda) : cb[u];
      }
    }
#pragma unroll
    for (int u = 0; u < kFullBatch; u++) {
      const int64_t j = base + (int64_t)u * kFullThreads;
      if (rw[u]) {
        A[b + j * lda] = y[u];
        A[pr + j * lda] = x[u];
      }
      if (cl[u]) {
        A[j + b * lda] = j > b ? mul_rn(cp[u], inv) : cp[u];
        if (pc != b) A[j + pc * lda] = cb[u];
      }
    }
  }
}

}  // namespace

// In-place full-pivoting elimination of the n x n matrix A (device,
// column-major, leading dimension lda).  rowpiv[k] / colpiv[k] (device, n
// int32) receive the row and column swapped into position k at step k (k
// itself for no swap or a skipped step); entry n - 1 is n - 1.
template <typename T>
int getrf_full_t(int64_t n, T *A, int64_t lda, int32_t *rowpiv,
                 int32_t *colpiv, T eps) {
  if (n <= 0) return 0;
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  cudaStream_t s = cx->stream;
  // one wave: as many CTAs as are resident at once on the current device,
  // striding over the tiles (queried per call: a cheap host query, and the
  // answer belongs to the device that is current now)
  int occ = 0;
  MGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &occ, lu_full_step_kernel<T>, kFullThreads, 0));
  if (occ < 1) occ = 1;
  const int64_t gmax = (int64_t)cx->sms * occ;
  const size_t part_bytes = (size_t)gmax * (sizeof(T) + 8);
  const size_t scratch = 256 + part_bytes + (size_t)n * 4;
  char *w = (char *)ws(WS_T0, scratch);
  if (!w) return MATGB_ERR_NOMEM;
  FullPivState *st = (FullPivState *)w;
  unsigned long long *part_r = (unsigned long long *)(w + 256);
  T *part_v = (T *)(w + 256 + (size_t)gmax * 8);
  int32_t *skip = (int32_t *)(w + 256 + part_bytes);
  MGB_CUDA(cudaMemsetAsync(w, 0, scratch, s));
  // Identity pivots: step n - 1 never runs, and n = 1 has no step.
  full_iota_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, 0,
                     s>>>(rowpiv, colpiv, n);
  MGB_LAUNCHED("full_iota");
  if (n == 1) return 0;
  for (int64_t k = -1; k + 1 < n; k++) {
    const int64_t m = n - k - 1;
    const int64_t tiles = ((m + kFullRows - 1) / kFullRows) *
                          ((m + kFullTileCols - 1) / kFullTileCols);
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, gmax);
    KtScope kt("lu_full_step", 2.0 * m * m, (k >= 0 ? 2.0 : 1.0) * sizeof(T) * m * m);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kFullThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    MGB_CUDA(cudaLaunchKernelEx(&cfg, lu_full_step_kernel<T>, A, n, lda, k, st,
                                part_v, part_r, rowpiv, colpiv, skip, eps));
    MGB_LAUNCHED("lu_full_step");
  }
  return 0;
}

template int getrf_full_t<float>(int64_t, float *, int64_t, int32_t *,
                                 int32_t *, float);
template int getrf_full_t<double>(int64_t, double *, int64_t, int32_t *,
                                  int32_t *, double);

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_getrf_full_dev(size_t n, mat_elem_t *A, size_t lda, int32_t *rowpiv,
                         int32_t *colpiv) {
  if (lda < n) return set_error(MATGB_ERR_ARG, "getrf_full: lda < n");
  if (n > 0 && (!rowpiv || !colpiv))
    return set_error(MATGB_ERR_ARG, "getrf_full: pivot arrays are NULL");
  if (n > 2147483647u) return set_error(MATGB_ERR_ARG, "getrf_full: n too large");
  return getrf_full_t<elem_t>((int64_t)n, A, (int64_t)lda, rowpiv, colpiv,
                              kPivotEps);
}

}  // extern "C"
