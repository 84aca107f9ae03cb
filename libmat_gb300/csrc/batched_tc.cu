// Mixed-precision batched solver on the tensor cores (float build): the
// systems of order 33..128 of a batched call (see batched.cu), each solved by
// one CTA with one thread per matrix row, refined to an FP32-level residual.
// It answers the same question as looping mat_solve / mat_solve_spd
// (mat.h:4807-4871) over the systems; it is a separate mode
// (matgb_batched_mixed), not the reference's operation order.
//
// Storage: the system's matrix lives in tensor memory (TMEM), row r in lane r,
// column c in TMEM column c (128 columns for orders 65..128, 64 for 33..64);
// thread r reads and writes its own lane with tcgen05.ld / tcgen05.st.
//
// Factorisation: blocked Gauss-Jordan in 32-column panels.  A panel's columns
// are loaded into registers; each thread keeps a 32-entry frame: before step
// j it holds its entries of panel columns j..31 followed by its row of the
// panel's transform so far (an augmented identity: the step that makes row p
// the pivot of column j starts column j of the transform at e_p), shifted
// left by one per step so every register index is static while the step loop
// is an ordinary loop.  Step j: the pivot row stages its frame, its
// right-hand side and its reciprocal in shared memory, one barrier, and every
// other row (rows above the pivot included: Gauss-Jordan) eliminates:
// frame[k] <- frame[k+1] - l * pivot_frame[k+1], frame[31] <- -l (the pivot
// row itself: 1).  After 32 steps the frame is the row of T[:, pivots], where
// T = I + W E^T is the panel's transform (E selects the 32 pivot rows), so
// W = frame - E.  The trailing columns then take T:
//   D[:, trailing] += W * P,   P = the pivot rows' trailing entries,
// one tcgen05.mma product with M = 128 (every row), N = trailing columns,
// K = 32, accumulating into the matrix in TMEM.  The operands are split into
// TF32 hi + remainder (hi = the value rounded to TF32, remainder = the exact
// FP32 difference), and Wh*Ph + Wh*Pl + Wl*Ph run as three products: ~21
// bits per product with FP32's exponent range (no scaling).  W itself stays
// in the panel's TMEM columns (they are finished) for the refinement solves.
// The right-hand side is eliminated with the panel steps, so after the last
// panel the pivot row of column c holds d_c x_c and no back substitution is
// needed.
//
// Pivoting (general systems): partial pivoting with mat_plu's rule on the
// values this factorisation computes (first logical row of max |a|; rows
// trade roles, not data; a pivot below eps is not eliminated with).  The
// kernel first takes row c as the pivot of column c with no search and checks
// that every row below would have lost the search (as the register kernel
// does); a system where a row would have won is factored again with the
// search.  SPD systems: the symmetric matrix rebuilt from the lower triangle,
// no exchanges, a pivot <= 0 gives status -1 (x untouched), as mat_chol.
//
// Refinement: r = b - A x with the original A (re-read; it is in L2) in FP32,
// eta = |r|inf / (|A|inf |x|inf + |b|inf); stop when eta <= n * 2^-24, else
// x += D^-1 T_P..T_1 r (per panel: the pivot rows publish their residuals,
// every row adds its W row times them -- matrix-vector work only), at most
// kBtMaxCorr corrections, or until eta stops halving.  status 0: converged;
// 1: not converged (x holds the last iterate).
#include "batched_kernels.cuh"
#include "tc_ptx.cuh"

namespace mgb {

#ifndef MAT_DOUBLE_PRECISION

constexpr int kBtP = 32;            // panel width (one K block of the MMA)
constexpr int kBtMaxCorr = 4;       // refinement corrections at most
constexpr uint32_t kBtWait = 2000000u;  // mbarrier polls (~0.2 s) before giving up
// the pivot-free pass is kept when every entry of its panel transforms is at
// most this large (GJ transform rows -(a_r / d) T_BB); otherwise the system is
// factored again with the pivot search
constexpr float kBtGrowth = 1.0f;

// Shared memory of one CTA.  aop: the A operand (W, 128 rows: the MMA's M),
// [hi: 128 rows x 128 B][remainder: 128 rows x 128 B], K-major with the
// 128-byte swizzle (16-byte chunk c of row r at chunk c ^ (r & 7)).  Rows at
// or above NT are never written: what the MMA reads there lands in TMEM lanes
// no thread owns, so for NT = 64 the B operand lives in those rows.  bop: the B operand, one 128-byte row per trailing column,
// [hi][remainder].
struct BtMisc {
  __align__(16) float hist[32][36];     // the pivot warp's 32 x 33 transposes
  __align__(16) float step[2][36];      // the pivot-free pass: a step's pivot frame, rb, 1/piv
  __align__(16) float stage[2][4][36];  // the search pass: per step parity and warp
  float bB[32];      // the pivot rows' right-hand sides before the panel
  float rcp[32];     // the panel's pivots' reciprocals
  unsigned wkey[2][4];
  int widx[2][4];
  float xs[128];     // the solution by logical column
  float gs[2][32];   // refinement: a panel's pivot-row residuals
  float red[2][4][2];
  int flag;
  int spdfail;
  int rshift;
  int take;
  uint32_t tmem;
  uint64_t mbar;
};

template <int NT>
struct BtLayout {
  static constexpr int kCols = NT <= 64 ? 64 : 128;  // TMEM columns
  static constexpr int kTrail = NT - kBtP;           // most trailing columns
  static constexpr int ahi = 0;
  static constexpr int alo = 16384;
  static constexpr int bhi = NT <= 64 ? 64 * 128 : 32768;
  static constexpr int blo = NT <= 64 ? 16384 + 64 * 128 : 32768 + kTrail * 128;
  static constexpr int misc = NT <= 64 ? 32768 : blo + kTrail * 128;
  static constexpr int bytes = (misc + (int)sizeof(BtMisc) > 32768 ? misc + (int)sizeof(BtMisc)
                                                                    : 32768);
  // resident CTAs per SM allowed by TMEM (512 columns)
  static constexpr int kMaxCtas = 512 / kCols;
};
static_assert(BtLayout<64>::blo + 32 * 128 <= 32768, "NT=64 bop lo overflows");

// Byte offset of element (row, k) (4-byte elements, K = 0..31) in a K-major
// 128-byte-swizzled operand.
__device__ __forceinline__ int sw_off(int row, int k) {
  return row * 128 + ((((k >> 2) ^ (row & 7))) << 4) + ((k & 3) << 2);
}

// TF32 hi part (round to nearest at the 10th fraction bit) and the exact FP32
// remainder.
__device__ __forceinline__ void tf32_split(float v, float &hi, float &lo) {
  hi = __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xffffe000u);
  lo = v - hi;
}

// Entry (r, c) of the system as the solver sees it: general systems read A;
// SPD systems mirror the lower triangle (all mat_chol reads).
template <int KIND>
__device__ __forceinline__ float bt_a(const float *__restrict__ A, int n, int r, int c) {
  if (KIND == 1 && c > r) return A[c + (int64_t)r * n];
  return A[r + (int64_t)c * n];
}

// Row t's entries of columns c0..c0+31 as stored (A[t + c n]; lanes along
// rows: coalesced), zero outside the system; one pointer stepped by n.
__device__ __forceinline__ void bt_row_direct(const float *__restrict__ A, int n, int t, int c0,
                                              float (&v)[32]) {
  const float *q = A + t + (int64_t)c0 * n;
  const bool rok = t < n;
#pragma unroll
  for (int k = 0; k < 32; k++, q += n) v[k] = (rok && c0 + k < n) ? *q : 0.f;
}

// Row t's entries of columns c0..c0+31 of an SPD system (the lower triangle
// mirrored), for the whole warp: entries at or below the diagonal are read
// directly (A[t + c n], lanes along rows: coalesced); entries above it are
// A[c + t n], read as the stored 32 x 32 tile with lanes along c (coalesced)
// and transposed through the warp's shared tile (32 x 33 floats).
__device__ __forceinline__ void bt_spd_chunk(const float *__restrict__ A, int n, int t, int c0,
                                             float (&v)[32], float *tile) {
  const int lane = t & 31, r0 = t - lane;
  if (c0 + 31 <= r0) {  // every entry at or below the diagonal
    bt_row_direct(A, n, t, c0, v);
    return;
  }
  {
    // the stored tile rows c0.., columns r0..: lane i holds row c0 + i
    float w[32];
    const float *q = A + (c0 + lane) + (int64_t)r0 * n;
    const bool rok = c0 + lane < n;
#pragma unroll
    for (int j = 0; j < 32; j++, q += n) w[j] = (rok && r0 + j < n) ? *q : 0.f;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 32; j++) tile[lane * 33 + j] = w[j];
    __syncwarp();
  }
  const bool diag = c0 < r0 + 32;  // the diagonal tile: entries c <= t direct
  const float *q = A + t + (int64_t)c0 * n;
#pragma unroll
  for (int k = 0; k < 32; k++, q += n) {
    const bool own = t < n && c0 + k < n;
    v[k] = own ? ((diag && c0 + k <= t) ? *q : tile[k * 33 + lane]) : 0.f;
  }
}

// Write row `row` of a K-major tensor-core operand (32 TF32 K entries, hi
// and remainder parts) from get(k), 16 bytes at a time.
template <class G>
__device__ __forceinline__ void bt_put_row(unsigned char *hi, unsigned char *lo, int row, G get) {
#pragma unroll
  for (int k = 0; k < 32; k += 4) {
    float h[4], r4[4];
#pragma unroll
    for (int e = 0; e < 4; e++) tf32_split(get(k + e), h[e], r4[e]);
    *reinterpret_cast<float4 *>(hi + sw_off(row, k)) = make_float4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<float4 *>(lo + sw_off(row, k)) = make_float4(r4[0], r4[1], r4[2], r4[3]);
  }
}

// D (TMEM, M = 128 rows, N columns) (+)= A * B^T with K = 32, as the three
// TF32 products Ah*Bh + Ah*Bl + Al*Bh (8 K entries, 32 bytes, per
// instruction).  Issued by one thread.
__device__ __forceinline__ void bt_mma(uint32_t d, int N, const unsigned char *ahi,
                                       const unsigned char *alo, const unsigned char *bhi,
                                       const unsigned char *blo, bool accumulate) {
  const uint32_t idesc = tc::idesc_tf32(128, N);
  const uint32_t a0 = tc::smem_u32(ahi), a1 = tc::smem_u32(alo);
  const uint32_t b0 = tc::smem_u32(bhi), b1 = tc::smem_u32(blo);
#pragma unroll
  for (int kk = 0; kk < 4; kk++) {
    tc::mma_tf32(d, tc::desc_k_sw128(a0 + kk * 32), tc::desc_k_sw128(b0 + kk * 32), idesc,
                 (accumulate || kk > 0) ? 1u : 0u);
    tc::mma_tf32(d, tc::desc_k_sw128(a0 + kk * 32), tc::desc_k_sw128(b1 + kk * 32), idesc, 1u);
    tc::mma_tf32(d, tc::desc_k_sw128(a1 + kk * 32), tc::desc_k_sw128(b0 + kk * 32), idesc, 1u);
  }
}

// Largest |v| over the CTA (v >= 0): warp redux on the bit patterns
// (non-negative floats order like their bits), one slot per warp; read after
// the next barrier with bt_max_read.
__device__ __forceinline__ void bt_max_post(float v, float *slot4, int warp) {
  const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(v));
  if ((threadIdx.x & 31) == 0) slot4[warp * 2] = __uint_as_float(m);
}

template <int NW>
__device__ __forceinline__ float bt_max_read(const float *slot4) {
  float m = slot4[0];
#pragma unroll
  for (int w = 1; w < NW; w++) m = fmaxf(m, slot4[w * 2]);
  return m;
}

// Wait (thread 0, bounded) for the last committed tensor-core product; the
// whole CTA learns the outcome at the barrier.  False: the wait gave up.
__device__ __forceinline__ bool bt_wait(BtMisc &m, int t, uint32_t ncommit) {
  if (t == 0) m.flag = tc::mbar_wait(&m.mbar, (ncommit - 1) & 1u, kBtWait, 256) ? 0 : 1;
  __syncthreads();
  tc::tc_fence_after();
  return m.flag == 0;
}

// One system.  Returns the status (0, 1, -1), or -3 when a wait for the
// tensor core gave up (the CTA then stops).
template <int NT, int KIND>
__device__ int bt_solve(const float *__restrict__ A, int n, const float *__restrict__ b,
                        float *__restrict__ x, unsigned char *sb, BtMisc &m,
                        uint32_t tbase, uint32_t &ncommit, float eps, int *ncorr, int rshift) {
  using L = BtLayout<NT>;
  constexpr int NW = NT / 32;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  // this thread's matrix row: the rows are rotated by whole warps per CTA
  // (rshift), so the pivot warps of CTAs sharing an SM sit on different
  // schedulers; row r lives in TMEM lane t
  const int r = (t + NT - rshift) % NT;
  const bool act = r < n;
  const uint32_t trow = tbase + ((uint32_t)(warp * 32) << 16);
  unsigned char *ahi = sb + L::ahi, *alo = sb + L::alo;
  unsigned char *bhi = sb + L::bhi, *blo = sb + L::blo;
  const int npan = (n + kBtP - 1) / kBtP;
  bool search = false;
  float rb = 0.f, dpiv = 1.f;
  int mycol = -1;

  for (;;) {  // a second pass with the pivot search if the first was beaten
    // ---- load: the rows into TMEM ---------------------------------------------
    float rowsum = 0.f;
    rb = act ? b[r] : 0.f;
    if (KIND == 1) {
      float *tile = reinterpret_cast<float *>(sb) + warp * (32 * 33);
#pragma unroll 1
      for (int c0 = 0; c0 < n; c0 += 32) {
        float v[32];
        bt_spd_chunk(A, n, r, c0, v, tile);
#pragma unroll
        for (int k = 0; k < 32; k++) rowsum += fabsf(v[k]);
        tc::tmem_st32(trow + (uint32_t)c0, v);
      }
    } else {
      // two 32-column chunks in flight
      auto load = [&](float (&v)[32], int c0) {
        bt_row_direct(A, n, r, c0, v);
#pragma unroll
        for (int k = 0; k < 32; k++) rowsum += fabsf(v[k]);
      };
      float va[32], vb[32];
      load(va, 0);
#pragma unroll 1
      for (int c0 = 0; c0 < n; c0 += 64) {
        if (c0 + 32 < n) load(vb, c0 + 32);
        tc::tmem_st32(trow + (uint32_t)c0, va);
        if (c0 + 32 < n) {
          if (c0 + 64 < n) load(va, c0 + 64);
          tc::tmem_st32(trow + (uint32_t)(c0 + 32), vb);
        }
      }
    }
    tc::tc_fence_before();
    bt_max_post(rowsum, &m.red[0][0][0], warp);      // |A|inf
    bt_max_post(fabsf(rb), &m.red[0][0][1], warp);   // |b|inf
    if (t == 0) m.spdfail = 0;  // read by the other warps after a barrier
    int lr = r;  // logical row played by this thread
    mycol = -1;
    dpiv = 1.f;
    bool beaten = false;
    int fail = 0;  // 1: SPD pivot <= 0; 2: beaten (search again)

    for (int p = 0; p < npan && !fail; p++) {
      const int c0 = p * kBtP;
      const int w = n - c0 < kBtP ? n - c0 : kBtP;
      const int ntr = n - c0 - kBtP;  // trailing columns
      if (p > 0) {
        // the previous panel's trailing update is complete
        if (!bt_wait(m, t, ncommit)) return -3;
      }
      float f[32];
      tc::tmem_ld32(trow + (uint32_t)c0, f);
      float W[32];  // this row of the panel's transform, T = I + W E^T
      bool bad = false;
      if (!search) {
        // ---- pivot-free pass ------------------------------------------------
        // The pivots are rows c0..c0+31, all in warp pw0.  That warp runs the
        // panel's 32 Gauss-Jordan steps on its own rows (warp-synchronous);
        // its frames end as T_BB, the transform's rows of the pivot block.
        // Every other row's transform row is then W_r = -(a_r / d) T_BB (a_r
        // its panel entries, d the pivots), one tensor-core product for all
        // rows at once.
        const int pw0 = ((c0 + rshift) >> 5) % NW;
        float *tile = &m.hist[0][0];  // the pivot warp's 32 x 33 transposes
        if (warp == pw0) {
          m.bB[lane] = rb;  // the pivot rows' right-hand sides before the panel
#pragma unroll 1
          for (int j = 0; j < w; j++) {
            const int c = c0 + j;
            float *h = m.step[j & 1];
            if (lane == j) {
              // the hardware reciprocal (~1 ulp): the mixed mode's factors are
              // approximate by design and the refinement measures the result
              const float rc = __fdividef(1.f, f[0]);
#pragma unroll
              for (int k = 0; k < 32; k += 4)
                *reinterpret_cast<float4 *>(h + k) = make_float4(f[k], f[k + 1], f[k + 2], f[k + 3]);
              *reinterpret_cast<float2 *>(h + 32) = make_float2(rb, rc);
              m.rcp[j] = rc;
            }
            __syncwarp();
            float uu[36];
#pragma unroll
            for (int k = 0; k < 36; k += 4) {
              const float4 q4 = *reinterpret_cast<const float4 *>(h + k);
              uu[k] = q4.x;
              uu[k + 1] = q4.y;
              uu[k + 2] = q4.z;
              uu[k + 3] = q4.w;
            }
            const float piv = uu[0];
            if (KIND == 1 && piv <= 0.f) {  // NaN passes, as in mat_chol
              if (lane == 0) m.spdfail = 1;
              break;
            }
            // within the block, partial pivoting must keep the diagonal (the
            // last column is not searched, as in mat_plu)
            if (KIND == 0 && act && lane > j && c < n - 1 && fabsf(f[0]) > fabsf(piv))
              beaten = true;  // (a NaN shows up in the transform check below)
            const bool is_piv = lane == j;
            const bool elim = KIND == 1 || !(fabsf(piv) < eps);
            float l = 0.f;
            if (is_piv) {
              dpiv = f[0];
              mycol = c;
            } else if (act && elim) {
              l = f[0] * uu[33];  // the pivot's reciprocal, computed once
            }
#pragma unroll
            for (int k = 0; k < 31; k++) f[k] = fmaf(-l, uu[k + 1], f[k + 1]);
            f[31] = is_piv ? 1.f : -l;
            rb = fmaf(-l, uu[32], rb);
          }
          // a short last panel: shift the transform's columns into place
#pragma unroll 1
          for (int j = w; j < kBtP; j++) {
#pragma unroll
            for (int k = 0; k < 31; k++) f[k] = f[k + 1];
            f[31] = 0.f;
          }
          // the product's B operand, T_BB^T (row = output column n, K = k),
          // transposed through the tile; the pivot rows' A operand rows are 0
#pragma unroll
          for (int k = 0; k < 32; k++) tile[lane * 33 + k] = f[k];
          __syncwarp();
          bt_put_row(bhi, blo, lane, [&](int k) { return tile[k * 33 + lane]; });
          bt_put_row(ahi, alo, t, [&](int) { return 0.f; });
        }
        __syncthreads();
        if (KIND == 1 && m.spdfail) {
          fail = 1;
          break;
        }
        if (warp != pw0) {
          // A operand: -(a_r / d) over the panel's columns
          bt_put_row(ahi, alo, t, [&](int k) { return k < w ? -f[k] * m.rcp[k] : 0.f; });
        }
        tc::fence_proxy_async_smem();
        tc::tc_fence_before();
        __syncthreads();
        if (t == 0) {
          tc::tc_fence_after();
          bt_mma(tbase + (uint32_t)c0, 32, ahi, alo, bhi, blo, false);
          tc::mma_commit(&m.mbar);
        }
        ncommit++;
        if (!bt_wait(m, t, ncommit)) return -3;
        if (warp == pw0) {
#pragma unroll
          for (int k = 0; k < 32; k++) W[k] = f[k] - (k == lane && lane < w ? 1.f : 0.f);
          tc::tmem_st32(trow + (uint32_t)c0, W);  // the product left 0 in these lanes
        } else {
          tc::tmem_ld32(trow + (uint32_t)c0, W);
          float acc = 0.f, wmax = 0.f;
#pragma unroll
          for (int k = 0; k < 32; k++) {
            acc = fmaf(W[k], m.bB[k], acc);
            wmax = fmaxf(wmax, fabsf(W[k]));
          }
          rb += acc;
          // a transform this large means the diagonal pivots are not safe:
          // factor again with the search (NaN included)
          if (KIND == 0 && !(wmax <= kBtGrowth)) bad = true;
        }
      } else {
        // ---- pass with the pivot search: one barrier per step ---------------
#pragma unroll 1
        for (int j = 0; j < w; j++) {
          const int c = c0 + j;
          const int par = j & 1;
          const bool cand = act && lr >= c;
          const unsigned key = cand ? fkey(f[0], lr == c) : 0u;
          const unsigned wk = __reduce_max_sync(0xffffffffu, key);
          const unsigned wi = __reduce_min_sync(
              0xffffffffu, (cand && key == wk) ? (unsigned)lr : 0x3fffffffu);
          if (lane == 0) {
            m.wkey[par][warp] = wk;
            m.widx[par][warp] = (int)((wi << 2) | (unsigned)warp);
          }
          const bool wbest = cand && (unsigned)lr == wi;
          if (wbest) {
            float *sg = m.stage[par][warp];
#pragma unroll
            for (int k = 0; k < 32; k += 4)
              *reinterpret_cast<float4 *>(sg + k) = make_float4(f[k], f[k + 1], f[k + 2], f[k + 3]);
            *reinterpret_cast<float2 *>(sg + 32) = make_float2(rb, __frcp_rn(f[0]));
          }
          __syncthreads();
          const unsigned ck = lane < NW ? m.wkey[par][lane] : 0u;
          const unsigned ci = lane < NW ? (unsigned)m.widx[par][lane] : 0xffffffffu;
          const unsigned bk = __reduce_max_sync(0xffffffffu, ck);
          const unsigned bi = __reduce_min_sync(0xffffffffu, ck == bk ? ci : 0xffffffffu);
          const int pl = (int)(bi >> 2);
          const int pw = (int)(bi & 3u);
          const bool is_piv = wbest && warp == pw;
          if (is_piv)
            lr = c;
          else if (act && lr == c)
            lr = pl;
          const float *u = m.stage[par][pw];
          float uu[36];
#pragma unroll
          for (int k = 0; k < 36; k += 4) {
            const float4 q4 = *reinterpret_cast<const float4 *>(u + k);
            uu[k] = q4.x;
            uu[k + 1] = q4.y;
            uu[k + 2] = q4.z;
            uu[k + 3] = q4.w;
          }
          const bool elim = !(fabsf(uu[0]) < eps);
          float l = 0.f;
          if (is_piv) {
            dpiv = f[0];
            mycol = c;
          } else if (act && elim) {
            l = f[0] * uu[33];
          }
#pragma unroll
          for (int k = 0; k < 31; k++) f[k] = fmaf(-l, uu[k + 1], f[k + 1]);
          f[31] = is_piv ? 1.f : -l;
          rb = fmaf(-l, uu[32], rb);
        }
#pragma unroll 1
        for (int j = w; j < kBtP; j++) {
#pragma unroll
          for (int k = 0; k < 31; k++) f[k] = f[k + 1];
          f[31] = 0.f;
        }
        // W = frame - E, kept in the panel's TMEM columns for the refinement
        const int jj = (mycol >= c0 && mycol < c0 + kBtP) ? mycol - c0 : -1;
#pragma unroll
        for (int k = 0; k < 32; k++) W[k] = f[k] - (k == jj ? 1.f : 0.f);
        tc::tmem_st32(trow + (uint32_t)c0, W);
      }

      // ---- the trailing update D[:, trailing] += W P ----------------------
      if (ntr > 0) {
        bt_put_row(ahi, alo, t, [&](int k) { return W[k]; });
        if (!search) {
          // the pivot rows are the lanes of warp pw0: their trailing entries
          // are transposed through the tile into one B row per column
          if (warp == ((c0 + rshift) >> 5) % NW) {
            float *tile = &m.hist[0][0];
            for (int q0 = 0; q0 < ntr; q0 += 32) {
              float v[32];
              tc::tmem_ld32(trow + (uint32_t)(c0 + kBtP + q0), v);
              __syncwarp();
#pragma unroll
              for (int i = 0; i < 32; i++) tile[lane * 33 + i] = v[i];
              __syncwarp();
              if (q0 + lane < ntr)
                bt_put_row(bhi, blo, q0 + lane, [&](int k) { return tile[k * 33 + lane]; });
            }
          }
        } else {
          // pivots anywhere: each pivot row scatters its entries (K = its step)
          const int jj = (mycol >= c0 && mycol < c0 + kBtP) ? mycol - c0 : -1;
          if (__any_sync(0xffffffffu, jj >= 0)) {
            for (int q0 = 0; q0 < ntr; q0 += 32) {
              float v[32];
              tc::tmem_ld32(trow + (uint32_t)(c0 + kBtP + q0), v);
              if (jj >= 0) {
#pragma unroll
                for (int i = 0; i < 32; i++) {
                  if (q0 + i < ntr) {
                    float h, r1;
                    tf32_split(v[i], h, r1);
                    *reinterpret_cast<float *>(bhi + sw_off(q0 + i, jj)) = h;
                    *reinterpret_cast<float *>(blo + sw_off(q0 + i, jj)) = r1;
                  }
                }
              }
            }
          }
        }
        // rows past the trailing columns up to the product's N are zero
        const int N = (ntr + 15) & ~15;
        if (t >= ntr && t < N) bt_put_row(bhi, blo, t, [&](int) { return 0.f; });
        tc::fence_proxy_async_smem();
        tc::tc_fence_before();
        if (__syncthreads_or(beaten || bad) != 0) {
          fail = 2;
          break;
        }
        if (t == 0) {
          tc::tc_fence_after();
          bt_mma(tbase + (uint32_t)(c0 + kBtP), N, ahi, alo, bhi, blo, true);
          tc::mma_commit(&m.mbar);
        }
        ncommit++;
      } else {
        tc::tc_fence_before();
        if (__syncthreads_or(beaten || bad) != 0) fail = 2;
      }
    }
    if (fail == 1) return -1;
    if (fail == 2) {
      // wait out the MMA already issued for this system (none is issued
      // after the check that failed), then factor again with the search
      search = true;
      __syncthreads();
      continue;
    }
    break;
  }

  // ---- solution and refinement ---------------------------------------------
  const float anorm = bt_max_read<NW>(&m.red[0][0][0]);
  const float bnorm = bt_max_read<NW>(&m.red[0][0][1]);
  float xv = mycol >= 0 ? rb / dpiv : 0.f;
  if (mycol >= 0) m.xs[mycol] = xv;
  __syncthreads();
  const float tol = (float)n * 5.9604645e-8f;  // n * 2^-24
  int st = 1;
  float eta_prev = INFINITY;
  for (int it = 0;; it++) {
    float rr = act ? b[r] : 0.f;
    {
      float p4[4] = {0.f, 0.f, 0.f, 0.f};
      float *tile = reinterpret_cast<float *>(sb) + warp * (32 * 33);
#pragma unroll 1
      for (int c0 = 0; c0 < n; c0 += 32) {
        float v[32];
        if (KIND == 1) {
          bt_spd_chunk(A, n, r, c0, v, tile);
        } else {
          bt_row_direct(A, n, r, c0, v);
        }
#pragma unroll
        for (int k = 0; k < 32; k++)
          if (c0 + k < n) p4[k & 3] = fmaf(v[k], m.xs[c0 + k], p4[k & 3]);
      }
      rr -= (p4[0] + p4[1]) + (p4[2] + p4[3]);
    }
    bt_max_post(fabsf(rr), &m.red[1][0][0], warp);
    bt_max_post(fabsf(xv), &m.red[1][0][1], warp);
    __syncthreads();
    const float rmax = bt_max_read<NW>(&m.red[1][0][0]);
    const float xmax = bt_max_read<NW>(&m.red[1][0][1]);
    __syncthreads();  // the slots are read before they are posted again
    const float den = anorm * xmax + bnorm;
    if (rmax <= tol * den) {  // also b = 0, x = 0
      st = 0;
      break;
    }
    const float eta = rmax / den;
    if (it == kBtMaxCorr || !(eta < 0.5f * eta_prev)) break;
    eta_prev = eta;
    if (t == 0 && ncorr) atomicAdd(ncorr, 1);
    // x += D^-1 T r: the panels' transforms in order
    for (int p = 0; p < npan; p++) {
      const int c0 = p * kBtP;
      const int g = p & 1;
      if (mycol >= c0 && mycol < c0 + kBtP) m.gs[g][mycol - c0] = rr;
      __syncthreads();
      float wrow[32];
      tc::tmem_ld32(trow + (uint32_t)c0, wrow);
      const int w = n - c0 < kBtP ? n - c0 : kBtP;
#pragma unroll
      for (int k = 0; k < 32; k++)
        if (k < w) rr = fmaf(wrow[k], m.gs[g][k], rr);
    }
    if (mycol >= 0) {
      xv += rr / dpiv;
      m.xs[mycol] = xv;
    }
    __syncthreads();
  }
  if (mycol >= 0) x[mycol] = xv;
  return st;
}

// Resident CTAs per SM the register allocator is asked for (the shared
// memory allows 3 / 4 / 6).
template <int NT>
struct BtMinCtas {
  static constexpr int v = NT == 128 ? 3 : NT == 96 ? 4 : 6;
};

template <int NT, int KIND>
__global__ void __launch_bounds__(NT, BtMinCtas<NT>::v)
    batched_tc_kernel(int queue, const int32_t *__restrict__ list, BatchQueues *q,
                      const int32_t *__restrict__ nvec, const int64_t *__restrict__ offA,
                      const float *__restrict__ A, const int64_t *__restrict__ offv,
                      const float *__restrict__ b, float *__restrict__ x,
                      int32_t *__restrict__ status, float eps) {
  using L = BtLayout<NT>;
  extern __shared__ __align__(1024) unsigned char bt_smem_raw[];
  // 1024-byte aligned by pointer arithmetic on the shared array, so every
  // access below stays a shared-memory access (an integer round trip would
  // make them generic)
  unsigned char *sb = bt_smem_raw + ((1024u - (tc::smem_u32(bt_smem_raw) & 1023u)) & 1023u);
  BtMisc &m = *reinterpret_cast<BtMisc *>(sb + L::misc);
  const int t = threadIdx.x, warp = t >> 5;
  if (t == 0) {
    tc::mbar_init(&m.mbar, 1);
    tc::fence_barrier_init();
  }
  if (warp == 0) tc::tmem_alloc(&m.tmem, L::kCols);
  if (t == 0) {
    // the CTA's first warp slot on the SM (warp slot % 4 is its scheduler):
    // rotate the rows so panel 0's pivot warp sits on scheduler
    // (CTA ordinal on the SM) % 4 where the rotation allows
    unsigned slot;
    asm volatile("mov.u32 %0, %%warpid;" : "=r"(slot));
    const int NW = NT / 32, k = (int)slot / NW;
    int sh = 0;
    for (int c = 0; c < NW; c++)
      if (((int)slot + c) % 4 == k % 4) {
        sh = c;
        break;
      }
    m.rshift = 32 * sh;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = m.tmem;
  const int rshift = m.rshift;
  int base = 0;
  for (int i = 0; i < queue; i++) base += q->count[i];
  const int cnt = q->count[queue];
  uint32_t ncommit = 0;
  bool dead = false;
  // systems are taken one ahead, so the next one's matrix is pulled towards
  // L2 while this one is solved
  if (t == 0) m.take = atomicAdd(&q->next[queue], 1);
  __syncthreads();
  int tk = m.take;
  for (;;) {
    if (tk >= cnt) break;
    __syncthreads();  // every thread has read m.take
    if (t == 0) m.take = atomicAdd(&q->next[queue], 1);
    __syncthreads();
    const int tn = m.take;
    if (tn < cnt && !dead) {
      const int s2 = list[base + tn];
      const int n2 = nvec[s2];
      if (n2 >= 1 && n2 <= NT) {
        const char *pa = reinterpret_cast<const char *>(A + offA[s2]);
        const int64_t lines = ((int64_t)n2 * n2 * 4 + 127) / 128;
        for (int64_t i = t; i < lines; i += NT) tc::prefetch_l2(pa + i * 128);
      }
    }
    const int s = list[base + tk];
    const int n = nvec[s];
    tk = tn;
    if (n < 1 || n > NT) continue;  // unsupported order: reported by the driver
    if (dead) {  // a wait gave up earlier: the rest of this CTA's systems are not solved
      if (t == 0) status[s] = -3;
      continue;
    }
    const int st = bt_solve<NT, KIND>(A + offA[s], n, b + offv[s], x + offv[s], sb, m,
                                      tbase, ncommit, eps, &q->tc_corr, rshift);
    if (t == 0) {
      status[s] = st;
      if (st == 1) atomicAdd(&q->tc_unconv, 1);
      if (st == -3) atomicExch(&q->tc_err, 1);
    }
    if (st == -3) dead = true;
  }
  // every issued product has completed (each system waits for its own
  // before its next panel; the last panel issues none) -- but a CTA that gave
  // up waits once more, bounded, before freeing TMEM
  if (dead && t == 0) tc::mbar_wait(&m.mbar, (ncommit - 1) & 1u, kBtWait, 0);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tbase, L::kCols);
}

template <int NT, int KIND>
static int launch_tc(int queue, const int32_t *list, BatchQueues *q, const int32_t *n,
                     const int64_t *offA, const float *A, const int64_t *offv,
                     const float *b, float *x, int32_t *status, int ctas_per_sm) {
  auto k = batched_tc_kernel<NT, KIND>;
  using L = BtLayout<NT>;
  // at least 1/(kMaxCtas+1) of the SM's shared memory, so the CTAs resident on
  // an SM never ask for more TMEM than it has (tcgen05.alloc would wait)
  const size_t floor_bytes = 233472 / (L::kMaxCtas + 1) + 1024;
  const size_t smem = (size_t)L::bytes + 1024 > floor_bytes ? (size_t)L::bytes + 1024 : floor_bytes;
  static bool attr = false;
  if (!attr) {
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // the whole carve-out as shared memory: with the default preference the
    // occupancy query (and the launch) gets one CTA per SM
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
    attr = true;
  }
  // resident CTAs per SM from the kernel's own resources (registers, shared
  // memory with the per-CTA reservation, TMEM columns); the runtime's
  // occupancy query answered 1 for these kernels, below what the hardware
  // schedules
  static int per_sm_max = 0;
  if (!per_sm_max) {
    cudaFuncAttributes fa;
    MGB_CUDA(cudaFuncGetAttributes(&fa, k));
    int dev = 0, smem_sm = 0, resv = 0;
    MGB_CUDA(cudaGetDevice(&dev));
    MGB_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    MGB_CUDA(cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev));
    const int regs_warp = ((fa.numRegs + 7) / 8) * 8 * 32;
    const int by_regs = 65536 / (regs_warp * (NT / 32));
    const int by_smem = smem_sm / (int)(smem + resv);
    int v = by_regs < by_smem ? by_regs : by_smem;
    if (v > L::kMaxCtas) v = L::kMaxCtas;
    per_sm_max = v;
  }
  int per_sm = per_sm_max;
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  if (per_sm < 1) return set_error(MATGB_ERR_CUDA, "batched_tc: kernel does not fit an SM");
  const int grid = ctx()->sms * per_sm;
  static const char *names[2][3] = {{"batched_tc_lu_64", "batched_tc_lu_96", "batched_tc_lu_128"},
                                    {"batched_tc_spd_64", "batched_tc_spd_96", "batched_tc_spd_128"}};
  KtScope kt(names[KIND][NT == 64 ? 0 : NT == 96 ? 1 : 2], 0.0, 0.0);
  k<<<grid, NT, smem, ctx()->stream>>>(queue, list, q, n, offA, A, offv, b, x, status,
                                        kPivotEps);
  MGB_LAUNCHED("batched_tc");
  return 0;
}

int batched_tc_bucket(int bucket, int kind, int queue, const int32_t *list, BatchQueues *q,
                      const int32_t *n, const int64_t *offA, const elem_t *A,
                      const int64_t *offv, const elem_t *b, elem_t *x, int32_t *status,
                      int ctas_per_sm) {
  switch (bucket * 2 + kind) {
    case 4: return launch_tc<64, 0>(queue, list, q, n, offA, A, offv, b, x, status, ctas_per_sm);
    case 5: return launch_tc<64, 1>(queue, list, q, n, offA, A, offv, b, x, status, ctas_per_sm);
    case 6: return launch_tc<96, 0>(queue, list, q, n, offA, A, offv, b, x, status, ctas_per_sm);
    case 7: return launch_tc<96, 1>(queue, list, q, n, offA, A, offv, b, x, status, ctas_per_sm);
    case 8: return launch_tc<128, 0>(queue, list, q, n, offA, A, offv, b, x, status, ctas_per_sm);
    case 9: return launch_tc<128, 1>(queue, list, q, n, offA, A, offv, b, x, status, ctas_per_sm);
    default: return set_error(MATGB_ERR_ARG, "batched_tc: bucket %d has no tensor-core kernel", bucket);
  }
}

#else  // the double build has no mixed-precision batched kernels

int batched_tc_bucket(int, int, int, const int32_t *, BatchQueues *, const int32_t *,
                      const int64_t *, const elem_t *, const int64_t *, const elem_t *,
                      elem_t *, int32_t *, int) {
  return set_error(MATGB_ERR_ARG, "the mixed batched solver is float-only");
}

#endif

}  // namespace mgb
