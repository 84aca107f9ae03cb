// Mixed-precision LU + iterative refinement (the GB300 extension of
// mat_solve, mat.h:4807-4837).
//
// Factorisation: FP32 panels and FP32 trailing matrix, with the trailing
// update A22 -= L21*U12 (mat.h:4277-4283) on the tensor cores: L21 and U12 are
// rounded to BF16 or FP16 once per 128-column block and multiplied by
// tc_gemm (FP32 accumulation in TMEM).  FP16 uses a per-block power-of-two
// scale of U12 (L21 is bounded by 1 under partial pivoting) so that small
// Schur-complement entries do not fall into FP16's subnormal range.
//
// Refinement: in the library's element type (FP64 in libmatgb_f64): the
// residual r = b - A x, the convergence test on the normwise backward error
// eta = |r|_inf / (|A|_inf |x|_inf + |b|_inf), and the update x += d run on
// the GPU in that precision; each correction d solves LU d = r / |r|_inf in
// FP32 with the low-precision factors.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <string.h>

#include <vector>

#include "internal.cuh"
#include "lp_pack.cuh"

#include <algorithm>

namespace mgb {

// ---- packing the trailing-update operands -------------------------------------
// to16 / from16 / fp16_scale: lp_pack.cuh.
// out[i*Kp + k] = A[i + k*lda] for i < m, k < nb (zero for nb <= k < Kp):
// L21 (column-major, M-contiguous) to a K-contiguous 16-bit operand.
// out_lo (optional): the remainder v - hi(v), also 16-bit (the split form).
template <int BF16>
__global__ void pack_l21_kernel(const float *__restrict__ A, int64_t lda,
                                int64_t m, int nb, int Kp,
                                uint16_t *__restrict__ out,
                                const unsigned *__restrict__ amax_bits,
                                float *__restrict__ scale,
                                uint16_t *__restrict__ out_lo = nullptr) {
  __shared__ float t[32][33];
  // optional FP16 scale s (products of two scaled operands carry s^2)
  const float s = amax_bits ? fp16_scale(*amax_bits) : 1.f;
  if (scale && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
    scale[0] = s;
    scale[1] = 1.f / s;
    scale[2] = 1.f / (s * s);
  }
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int64_t i0 = (int64_t)blockIdx.x * 32;
  const int k0 = blockIdx.y * 32;
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + tx;
    const int k = k0 + r;
    t[r][tx] = (i < m && k < nb) ? s * A[i + (int64_t)k * lda] : 0.f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + r;
    if (i < m) {
      const float v = t[tx][r];
      const uint16_t h = to16<BF16>(v);
      out[i * Kp + k0 + tx] = h;
      if (out_lo) out_lo[i * Kp + k0 + tx] = to16<BF16>(v - from16<BF16>(h));
    }
  }
}

// max |A(0:rows, 0:cols)| (column-major, leading dimension lda) into
// *amax_bits (atomicMax on the bit pattern: non-negative floats order like
// their bits).  A warp takes a (column, 1024-row chunk) task at a time, lanes
// down the column; NaN is ignored here and propagates through the GEMM.
__global__ void amax_kernel(const float *__restrict__ A, int64_t lda, int rows,
                            int64_t cols, unsigned *__restrict__ amax_bits) {
  const int lane = threadIdx.x & 31;
  const int nchunk = (rows + 1023) >> 10;
  const int64_t ntask = cols * nchunk;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  float m = 0.f;
  for (int64_t t = w0; t < ntask; t += nw) {
    const int64_t j = t / nchunk;
    const int r0 = (int)(t - j * nchunk) << 10;
    const int r1 = r0 + 1024 < rows ? r0 + 1024 : rows;
    const float *c = A + j * lda;
    for (int k = r0 + lane; k < r1; k += 32) m = fmaxf(m, fabsf(c[k]));
  }
  for (int off = 16; off; off >>= 1) m = fmaxf(m, __shfl_xor_sync(~0u, m, off));
  if (lane == 0) atomicMax(amax_bits, __float_as_uint(m));
}

// out[j*Kp + k] = s * A[k + j*lda] (k < nb), 0 for nb <= k < Kp, with
// s = fp16_scale(*amax_bits) (FP16) or 1 (BF16, or no amax).
// scale[1] = 1/s, or 1/(s * sL) when the L21 operand was scaled by
// sL = fp16_scale(*amax_l); out_lo (optional) gets the remainders.  A warp per
// column, two values per lane in one 32-bit store.
template <int BF16>
__global__ void pack_u12_kernel(const float *__restrict__ A, int64_t lda,
                                int nb, int Kp, int64_t ncols,
                                const unsigned *__restrict__ amax_bits,
                                float *__restrict__ scale,
                                uint16_t *__restrict__ out,
                                uint16_t *__restrict__ out_lo = nullptr,
                                const unsigned *__restrict__ amax_l = nullptr) {
  const float s = (!BF16 && amax_bits) ? fp16_scale(*amax_bits) : 1.f;
  if (blockIdx.x == 0 && threadIdx.x == 0 && scale) {
    const float sl = amax_l ? fp16_scale(*amax_l) : 1.f;
    scale[0] = s;
    scale[1] = 1.f / (s * sl);  // powers of two: exact
  }
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = w0; j < ncols; j += nw) {
    const float *c = A + j * lda;
    uint32_t *o = reinterpret_cast<uint32_t *>(out + j * Kp);
    uint32_t *ol = out_lo ? reinterpret_cast<uint32_t *>(out_lo + j * Kp) : nullptr;
    for (int k = 2 * lane; k < Kp; k += 64) {
      const float v0 = k < nb ? s * c[k] : 0.f;
      const float v1 = k + 1 < nb ? s * c[k + 1] : 0.f;
      const uint16_t h0 = to16<BF16>(v0), h1 = to16<BF16>(v1);
      o[k >> 1] = (uint32_t)h0 | ((uint32_t)h1 << 16);
      if (ol) {
        const uint16_t l0 = to16<BF16>(v0 - from16<BF16>(h0));
        const uint16_t l1 = to16<BF16>(v1 - from16<BF16>(h1));
        ol[k >> 1] = (uint32_t)l0 | ((uint32_t)l1 << 16);
      }
    }
  }
}

static unsigned grid_cap(int64_t tot, int per = 256) {
  int64_t b = (tot + per - 1) / per;
  int64_t cap = (int64_t)ctx()->sms * 16;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// lp: 1 BF16, 0 FP16 (U12 scaled by a power of two), 2 FP16 split (both
// operands scaled and split into hi + remainder; three tensor-core products).
// first: the block's first call -- L21 is packed (and, for the split, its
// scale found); every call packs the U12 columns [c0, c1) it updates, with a
// scale of its own (kept in a slot per call, so the two calls of a block --
// the look-ahead columns, then the rest -- never share one).
// amax3 (may be null): the block's three max slots -- |L21|, |U12| of the
// look-ahead columns, |U12| of the rest -- zeroed once per factorisation;
// l21_ready / u12_ready: the factorisation kernels already filled them.
// Without amax3 the maxima are found here in a zeroed scratch slot.
int lp_trailing_update(int64_t n, float *A, int64_t lda, int64_t kb,
                       int64_t ke, int64_t c0, int64_t c1, int lp, bool first,
                       unsigned *amax3, bool l21_ready, bool u12_ready, int wset) {
  const int nb = (int)(ke - kb);
  const int Kp = (nb + 63) / 64 * 64;
  const int64_t m = n - ke, ncols = n - ke, nc = c1 - c0;
  const bool split = lp == 2;
  const size_t an = (size_t)m * Kp, bn_ = (size_t)ncols * Kp;
  const int s0 = wset == 0 ? WS_T0 : WS_CU0 + 3 * (wset - 1);
  const int s1 = wset == 0 ? WS_T1 : s0 + 1, s2 = wset == 0 ? WS_T2 : s0 + 2;
  if (wset < 0 || wset > 8) return set_error(MATGB_ERR_ARG, "lp_trailing_update: bad set");
  uint16_t *A16 = (uint16_t *)ws(s0, an * 2 * (split ? 2 : 1));
  uint16_t *B16 = (uint16_t *)ws(s1, bn_ * 2 * (split ? 2 : 1));
  float *scb = (float *)ws(s2, 256);
  if (!A16 || !B16 || !scb) return MATGB_ERR_NOMEM;
  uint16_t *A16lo = split ? A16 + an : nullptr;
  uint16_t *B16lo = split ? B16 + bn_ : nullptr;
  // slots: [0..3] scales of the first call, [8..11] of the second;
  // [16] amax of L21 (split), [17], [18] amax of each call's U12 columns
  float *sc = scb + (first ? 0 : 8);
  unsigned *amax_l = amax3 ? amax3 : (unsigned *)(scb + 16);
  unsigned *amax_u = amax3 ? amax3 + (first ? 1 : 2) : (unsigned *)(scb + (first ? 17 : 18));
  if (!amax3) l21_ready = u12_ready = false;
  cudaStream_t st = ctx()->stream;
  const int64_t off = (c0 - ke) * Kp;
  {
    KtScope kt("lp_pack", 0.0,
               (split ? 10.0 : 6.0) * ((first ? m : 0) + nc) * nb);
    const float *L21 = A + ke + kb * lda;
    const float *U12 = A + kb + c0 * lda;
    if (lp != 1 && !u12_ready) {
      if (!amax3) MGB_CUDA(cudaMemsetAsync(amax_u, 0, sizeof(unsigned), st));
      amax_kernel<<<grid_cap(32 * nc), 256, 0, st>>>(U12, lda, nb, nc, amax_u);
      MGB_LAUNCHED("u12_amax");
    }
    if (first) {
      dim3 g((unsigned)((m + 31) / 32), (unsigned)(Kp / 32));
      if (split) {
        if (!l21_ready) {
          if (!amax3) MGB_CUDA(cudaMemsetAsync(amax_l, 0, sizeof(unsigned), st));
          amax_kernel<<<grid_cap(32 * (int64_t)nb * ((m + 1023) / 1024)), 256, 0, st>>>(
              L21, lda, (int)m, nb, amax_l);
          MGB_LAUNCHED("l21_amax");
        }
        pack_l21_kernel<0><<<g, 256, 0, st>>>(L21, lda, m, nb, Kp, A16, amax_l,
                                              nullptr, A16lo);
      } else if (lp == 1) {
        pack_l21_kernel<1><<<g, 256, 0, st>>>(L21, lda, m, nb, Kp, A16,
                                              nullptr, nullptr);
      } else {
        pack_l21_kernel<0><<<g, 256, 0, st>>>(L21, lda, m, nb, Kp, A16,
                                              nullptr, nullptr);
      }
      MGB_LAUNCHED("pack_l21");
    }
    if (lp == 1)
      pack_u12_kernel<1><<<grid_cap(32 * nc), 256, 0, st>>>(
          U12, lda, nb, Kp, nc, nullptr, sc, B16 + off);
    else
      pack_u12_kernel<0><<<grid_cap(32 * nc), 256, 0, st>>>(
          U12, lda, nb, Kp, nc, amax_u, sc, B16 + off,
          split ? B16lo + off : nullptr, split ? amax_l : nullptr);
    MGB_LAUNCHED("pack_u12");
  }
  return tc_gemm(lp == 1, m, nc, Kp, A16, Kp, B16 + off, Kp, -1.f,
                 lp != 1 ? sc + 1 : nullptr, 1.f, A + ke + c0 * lda, lda, 0,
                 nullptr, A16lo, split ? B16lo + off : nullptr);
}

// Cholesky: C22 (lower) -= L21 L21^T with L21 packed once to 16 bits and used
// as both operands; FP16 scales L21 by a power of two s and the epilogue
// multiplies by 1/s^2; the split form (lp 2) also packs the remainders.
// lp_syrk_pack packs into buffer set `set` (0 or 1, so that a look-ahead can
// pack the next block's operand while the current one is still read);
// lp_syrk_apply runs C (lower, relative to C's origin) -= rows [r0, r0+M)
// of the operand times rows [c0, c0+N) transposed.
// The max slot of set s (zeroed and filled by the Cholesky's own kernels
// when amax_ready).
unsigned *lp_syrk_amax_slot(int set) {
  float *sc = (float *)ws(set == 0 ? WS_T2 : WS_CU0 + 2, 64);
  return sc ? reinterpret_cast<unsigned *>(sc + 4) : nullptr;
}

int lp_syrk_pack(int64_t m, int nb, const float *L21, int64_t lda, int lp, int set,
                 SyrkOperand *op, bool amax_ready) {
  const int Kp = (nb + 63) / 64 * 64;
  const bool split = lp == 2;
  const size_t an = (size_t)m * Kp;
  const int s0 = set == 0 ? WS_T0 : WS_CU0, s2 = set == 0 ? WS_T2 : WS_CU0 + 2;
  uint16_t *A16 = (uint16_t *)ws(s0, an * 2 * (split ? 2 : 1));
  float *sc = (float *)ws(s2, 64);
  if (!A16 || !sc) return MATGB_ERR_NOMEM;
  op->hi = A16;
  op->lo = split ? A16 + an : nullptr;
  op->sc = sc;
  op->Kp = Kp;
  op->m = m;
  op->lp = lp;
  unsigned *amax = (unsigned *)(sc + 4);
  cudaStream_t st = ctx()->stream;
  KtScope kt("lp_pack", 0.0, (split ? 8.0 : 6.0) * m * nb);
  dim3 g((unsigned)((m + 31) / 32), (unsigned)(Kp / 32));
  if (lp == 1) {
    pack_l21_kernel<1><<<g, 256, 0, st>>>(L21, lda, m, nb, Kp, A16, nullptr, sc);
  } else {
    if (!amax_ready) {
      MGB_CUDA(cudaMemsetAsync(amax, 0, sizeof(unsigned), st));
      amax_kernel<<<grid_cap(32 * (int64_t)nb * ((m + 1023) / 1024)), 256, 0, st>>>(
          L21, lda, (int)m, nb, amax);
      MGB_LAUNCHED("l21_amax");
    }
    pack_l21_kernel<0><<<g, 256, 0, st>>>(L21, lda, m, nb, Kp, A16, amax, sc, op->lo);
  }
  MGB_LAUNCHED("pack_l21");
  return 0;
}

int lp_syrk_apply(const SyrkOperand &op, int64_t r0, int64_t M, int64_t c0, int64_t N,
                  float *C, int64_t ldc, const int32_t *info, int persist) {
  if (M <= 0 || N <= 0) return 0;
  const int64_t Kp = op.Kp;
  return tc_gemm(op.lp == 1, M, N, Kp, op.hi + r0 * Kp, Kp, op.hi + c0 * Kp, Kp, -1.f,
                 op.lp != 1 ? op.sc + 2 : nullptr, 1.f, C, ldc, 1, info,
                 op.lo ? op.lo + r0 * Kp : nullptr, op.lo ? op.lo + c0 * Kp : nullptr,
                 nullptr, nullptr, nullptr, nullptr, persist);
}

int lp_syrk_update(int64_t m, int nb, const float *L21, int64_t lda,
                   float *C22, int64_t ldc, int lp, const int32_t *info) {
  SyrkOperand op;
  MGB_TRY(lp_syrk_pack(m, nb, L21, lda, lp, 0, &op));
  return lp_syrk_apply(op, 0, m, 0, m, C22, ldc, info);
}

// ---- refinement kernels ------------------------------------------------------------
// W = (float)A (n x n), and, when rowsum is given, rowsum[i] += sum |A(i,j)|
// over the thread's chunk of columns: the one pass over A that the
// factorisation needs anyway also yields |A|_inf.  Thread = row, grid.y =
// column chunk (coalesced down each column).
template <typename S>
__global__ void to_float_rowsum_kernel(int64_t n, const S *__restrict__ A,
                                       int64_t lda, float *__restrict__ W,
                                       int64_t ldw, double *__restrict__ rowsum,
                                       int chunk, int64_t ncols) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t j0 = (int64_t)blockIdx.y * chunk;
  const int64_t j1 = j0 + chunk < ncols ? j0 + chunk : ncols;
  double s = 0;
#pragma unroll 8
  for (int64_t j = j0; j < j1; j++) {
    const S v = A[i + j * lda];
    W[i + j * ldw] = (float)v;
    s += fabs((double)v);
  }
  if (rowsum) atomicAdd(&rowsum[i], s);
}

// out = max_i rowsum[i] as the bit pattern of a non-negative double
// (monotone as an unsigned integer; NaN propagates as the largest pattern).
__global__ void rowmax_kernel(int64_t n, const double *__restrict__ rowsum,
                              unsigned long long *__restrict__ out) {
  unsigned long long m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(rowsum[i]);
    m = b > m ? b : m;
  }
  for (int off = 16; off; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, m, off);
    m = o > m ? o : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Per-column max |R(:,c)| and max |X(:,c)| (bit patterns of non-negative
// doubles; NaN propagates).  grid.y = column.
template <typename S>
__global__ void col_amax2_kernel(int64_t n, const S *__restrict__ R,
                                 int64_t ldr, const S *__restrict__ X,
                                 int64_t ldx,
                                 unsigned long long *__restrict__ out) {
  const int64_t c = blockIdx.y;
  double mr = 0, mx = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double a = fabs((double)R[i + c * ldr]), b = fabs((double)X[i + c * ldx]);
    mr = (a > mr || a != a) ? a : mr;
    mx = (b > mx || b != b) ? b : mx;
  }
  for (int off = 16; off; off >>= 1) {
    const double o1 = __shfl_xor_sync(~0u, mr, off);
    const double o2 = __shfl_xor_sync(~0u, mx, off);
    mr = (o1 > mr || o1 != o1) ? o1 : mr;
    mx = (o2 > mx || o2 != o2) ? o2 : mx;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out + 2 * c, (unsigned long long)__double_as_longlong(mr));
    atomicMax(out + 2 * c + 1, (unsigned long long)__double_as_longlong(mx));
  }
}

// RF(:,c) = R(:,c) / rn_c in FP32 (rn_c = out[2c], 1 when zero or not finite)
template <typename S>
__global__ void scale_to_float_kernel(int64_t n, const S *__restrict__ R,
                                      int64_t ldr,
                                      const unsigned long long *__restrict__ rn,
                                      float *__restrict__ RF) {
  const int64_t c = blockIdx.y;
  double s = __longlong_as_double((long long)rn[2 * c]);
  s = (s > 0 && s < INFINITY) ? 1.0 / s : 1.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    RF[i + c * n] = (float)((double)R[i + c * ldr] * s);
}

// max |v| over the block's threads into *out (double bits; NaN wins)
__device__ __forceinline__ void amax_into(double v, unsigned long long *out) {
  for (int off = 16; off; off >>= 1) {
    const double o = __shfl_xor_sync(~0u, v, off);
    v = (o > v || o != o) ? o : v;
  }
  if ((threadIdx.x & 31) == 0)
    atomicMax(out, (unsigned long long)__double_as_longlong(v));
}

// X(:,c) += rn_c * D(:,c); dn[c] = max |rn_c * D(:,c)| (the applied
// correction's size, the refinement's forward-error estimate)
template <typename S>
__global__ void update_x_kernel(int64_t n, S *__restrict__ X, int64_t ldx,
                                const float *__restrict__ D,
                                const unsigned long long *__restrict__ rn,
                                unsigned long long *__restrict__ dn) {
  const int64_t c = blockIdx.y;
  double s = __longlong_as_double((long long)rn[2 * c]);
  if (!(s > 0 && s < INFINITY)) s = 1.0;
  double md = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double d = s * (double)D[i + c * n];
    X[i + c * ldx] = (S)((double)X[i + c * ldx] + d);
    const double a = fabs(d);
    md = (a > md || a != a) ? a : md;
  }
  amax_into(md, dn + c);
}

template <typename S>
__global__ void copy_cols_kernel(int64_t n, int64_t nrhs, const S *__restrict__ B,
                                 int64_t ldb, S *__restrict__ R, int64_t ldr) {
  const int64_t tot = n * nrhs;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x)
    R[(e % n) + (e / n) * ldr] = B[(e % n) + (e / n) * ldb];
}

// X += D (element type); *dn = max |D|
template <typename S>
__global__ void add_vec_kernel(int64_t n, S *__restrict__ X,
                               const S *__restrict__ D,
                               unsigned long long *__restrict__ dn) {
  double md = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    X[i] = X[i] + D[i];
    const double a = fabs((double)D[i]);
    md = (a > md || a != a) ? a : md;
  }
  amax_into(md, dn);
}

// Reduced doubles (stored as bit patterns) to the host.
static int fetch(const unsigned long long *d, double *v, int count) {
  MGB_CUDA(cudaMemcpyAsync(v, d, count * sizeof(double), cudaMemcpyDeviceToHost,
                           ctx()->stream));
  MGB_CUDA(cudaStreamSynchronize(ctx()->stream));
  return 0;
}

struct IrEvents {
  cudaEvent_t e[3];
  bool ready = false;
};
static IrEvents g_ir;

// Solve A X = B (A n x n, B/X n x nrhs, column-major, library element type)
// with a low-precision LU (spd = false) or Cholesky (spd = true) and
// refinement in the element type.  Returns 0, or sets *not_spd when even the
// FP32 Cholesky meets a non-positive pivot.
// Residuals by digit slices on the tensor cores from this order up (below
// it the FP64 GEMM is cheap); matgb_resid64_mode switches them off.
constexpr int64_t kResid64MinN = 1024;
static int g_resid64_on = 1;

// Copy stream and events for a matrix that arrives from the host in column
// chunks while the factorisation runs (ArrivalPlan).
struct ArrivalRes {
  cudaStream_t cs = nullptr;
  cudaEvent_t start = nullptr;
  cudaEvent_t ev[kMaxChunks] = {};
  bool ready = false;
};
static ArrivalRes g_arr;
// From this order up a host matrix is copied in chunks under the
// factorisation (below it the copy is short).
constexpr int64_t kArrivalMinN = 8192;

static int arrival_setup() {
  if (g_arr.ready) return 0;
  MGB_CUDA(cudaStreamCreateWithFlags(&g_arr.cs, cudaStreamNonBlocking));
  MGB_CUDA(cudaEventCreateWithFlags(&g_arr.start, cudaEventDisableTiming));
  for (auto &e : g_arr.ev) MGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  g_arr.ready = true;
  return 0;
}

int solve_ir(bool spd, int64_t n, int64_t nrhs, const elem_t *A, int64_t lda,
             const elem_t *B, int64_t ldb, elem_t *X, int64_t ldx,
             const MatIROpts &o, MatIRReport *rep, int *not_spd,
             const elem_t *hA = nullptr) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (not_spd) *not_spd = 0;
  if (n <= 0 || nrhs <= 0) return 0;
  if (o.lp_format < -1 || o.lp_format > 3)
    return set_error(MATGB_ERR_ARG,
                     "lp_format must be 3 (three-part FP16 split), 2 (FP16 split), 1 "
                     "(BF16), 0 (FP16) or -1 (FP32)");
  if (!g_ir.ready) {
    for (auto &e : g_ir.e) MGB_CUDA(cudaEventCreate(&e));
    g_ir.ready = true;
  }
  cudaStream_t st = cx->stream;
  float *W = (float *)ws(WS_U, (size_t)n * n * sizeof(float));
  int32_t *piv = (int32_t *)ws(WS_PIV, (size_t)(2 * n + 8) * sizeof(int32_t));
  elem_t *R = (elem_t *)ws(WS_V0, (size_t)n * nrhs * sizeof(elem_t));
  float *RF = (float *)ws(WS_V1, (size_t)2 * n * nrhs * sizeof(float));
  unsigned long long *red = (unsigned long long *)ws(
      WS_INFO, (size_t)(3 * nrhs + 8) * sizeof(unsigned long long));
  if (!W || !piv || !R || !RF || !red) return MATGB_ERR_NOMEM;
  float *DF = RF + n * nrhs;
  int32_t *info = piv + 2 * n;
  unsigned long long *rs = red + 8;  // 2 per column
  unsigned long long *dn = rs + 2 * nrhs;  // 1 per column: last correction
  const dim3 cg(grid_cap(n) < 64 ? grid_cap(n) : 64, (unsigned)nrhs);
  const unsigned gnn = grid_cap(n * nrhs);

  // per-column |B|_inf now; |A|_inf from the first conversion of A
  double *rowsum = (double *)ws(WS_RS, (size_t)n * sizeof(double));
  if (!rowsum) return MATGB_ERR_NOMEM;
  MGB_CUDA(cudaMemsetAsync(red, 0, (size_t)(2 * nrhs + 8) * sizeof(unsigned long long), st));
  MGB_CUDA(cudaMemsetAsync(rowsum, 0, (size_t)n * sizeof(double), st));
  col_amax2_kernel<elem_t><<<cg, 256, 0, st>>>(n, B, ldb, B, ldb, rs);
  MGB_LAUNCHED("col_amax");
  std::vector<double> hv(3 * nrhs + 8);
  double anorm = 0;
  std::vector<double> bn(nrhs);
  const double eps = sizeof(elem_t) == 8 ? 1.1102230246251565e-16
                                         : 5.960464477539063e-08;
  const double tol = o.tol > 0 ? o.tol : (double)n * eps;
  const int maxit = o.max_iter > 0 ? o.max_iter : 100;

  // the three-part split is an LU form (the Cholesky takes the two-part one)
  int lp = spd && o.lp_format == 3 ? 2 : o.lp_format;
  double eta = INFINITY, rn = 0, xn = 0, fwd = INFINITY;
  int it = 0, converged = 0, refinements = 0, ksteps = 0;
  const bool use_krylov = o.krylov != 0 && nrhs == 1;
  const int kdim = o.krylov_dim > 0 ? (o.krylov_dim < kKrylovMaxDim ? o.krylov_dim
                                                                    : kKrylovMaxDim)
                                    : 50;
  float ms_factor = 0.f;
  for (int attempt = 0; attempt < 2; attempt++) {
    MGB_CUDA(cudaEventRecord(g_ir.e[0], st));
    constexpr int kChunk = 64;
    ArrivalPlan plan;
    const ArrivalPlan *pl = nullptr;
    if (hA && attempt == 0) {
      // the host matrix: copied in column chunks on a copy stream (into A,
      // which the refinement's residuals read) and converted to FP32 chunk by
      // chunk; the LU starts on the first chunk (ArrivalPlan)
      MGB_TRY(arrival_setup());
      constexpr int64_t blk = 144;  // the float LU's outer block
      int64_t cw = n;
      if (!spd && n >= kArrivalMinN && lda == n) {
        // four chunks: the LU starts after a quarter of the copy (measured at
        // n = 16384: mat_solve_ir 68.7 ms with four chunks, 76.3 ms with
        // eight -- each chunk's catch-up re-packs every finished block's L21 --
        // and 74.5 ms with the whole copy first)
        cw = (n / 4) / blk * blk;
        if (cw < 8 * blk) cw = 8 * blk;
      }
      plan.cw = cw;
      plan.nchunks = (int)((n + cw - 1) / cw);
      MGB_CUDA(cudaEventRecord(g_arr.start, st));
      MGB_CUDA(cudaStreamWaitEvent(g_arr.cs, g_arr.start, 0));
      for (int k = 0; k < plan.nchunks; k++) {
        const int64_t c0 = (int64_t)k * cw, c1 = c0 + cw < n ? c0 + cw : n;
        MGB_CUDA(cudaMemcpyAsync(const_cast<elem_t *>(A) + c0 * lda, hA + c0 * n,
                                 (size_t)(n * (c1 - c0)) * sizeof(elem_t),
                                 cudaMemcpyHostToDevice, g_arr.cs));
        const dim3 g((unsigned)((n + 255) / 256), (unsigned)((c1 - c0 + kChunk - 1) / kChunk));
        to_float_rowsum_kernel<elem_t><<<g, 256, 0, g_arr.cs>>>(
            n, A + c0 * lda, lda, W + c0 * n, n, rowsum, kChunk, c1 - c0);
        MGB_LAUNCHED("to_float");
        plan.ev[k] = g_arr.ev[k];
        MGB_CUDA(cudaEventRecord(plan.ev[k], g_arr.cs));
      }
      pl = &plan;
      if (spd)  // the Cholesky takes the whole matrix
        for (int k = 0; k < plan.nchunks; k++) MGB_CUDA(cudaStreamWaitEvent(st, plan.ev[k], 0));
    } else {
      const dim3 g((unsigned)((n + 255) / 256), (unsigned)((n + kChunk - 1) / kChunk));
      to_float_rowsum_kernel<elem_t><<<g, 256, 0, st>>>(
          n, A, lda, W, n, attempt == 0 ? rowsum : nullptr, kChunk, n);
      MGB_LAUNCHED("to_float");
    }
    if (attempt == 0 && !pl) {
      rowmax_kernel<<<grid_cap(n), 256, 0, st>>>(n, rowsum, red);
      MGB_LAUNCHED("rowmax");
    }
    if (spd)
      MGB_TRY(potrf_t<float>(n, W, n, info, lp));
    else
      MGB_TRY(getrf_t<float>(n, W, n, piv, piv + n, 0.f, lp, pl));
    if (pl) {
      // every chunk is in (the LU joined them all); then |A|inf
      for (int k = 0; k < plan.nchunks; k++) MGB_CUDA(cudaStreamWaitEvent(st, plan.ev[k], 0));
      rowmax_kernel<<<grid_cap(n), 256, 0, st>>>(n, rowsum, red);
      MGB_LAUNCHED("rowmax");
    }
    MGB_CUDA(cudaEventRecord(g_ir.e[1], st));
    MGB_CUDA(cudaEventSynchronize(g_ir.e[1]));
    if (attempt == 0) {
      MGB_TRY(fetch(red, hv.data(), 2 * (int)nrhs + 8));
      anorm = hv[0];
      for (int64_t c = 0; c < nrhs; c++) bn[c] = hv[8 + 2 * c];
    }
    float f = 0.f;
    cudaEventElapsedTime(&f, g_ir.e[0], g_ir.e[1]);
    ms_factor += f;
    if (spd) {
      int32_t hinfo = 0;
      MGB_CUDA(cudaMemcpy(&hinfo, info, sizeof hinfo, cudaMemcpyDeviceToHost));
      if (hinfo != 0) {  // the rounded matrix is not positive definite
        if (lp >= 0 && o.fp32_fallback) {
          lp = -1;
          continue;
        }
        if (not_spd) *not_spd = 1;
        break;
      }
    }

    MGB_CUDA(cudaMemsetAsync(red, 0, 8 * sizeof(unsigned long long), st));
    copy_cols_kernel<elem_t><<<gnn, 256, 0, st>>>(n, nrhs, B, ldb, R, n);
    MGB_LAUNCHED("copy_cols");
    for (int64_t c = 0; c < nrhs; c++)
      MGB_CUDA(cudaMemsetAsync(X + c * ldx, 0, (size_t)n * sizeof(elem_t), st));
    double prev = INFINITY;
    if (use_krylov) {
      // FGMRES cycles on the correction equation, residual in V(:, 0)
      elem_t *V = (elem_t *)ws(WS_KV, (size_t)(2 * kdim + 2) * n * sizeof(elem_t));
      if (!V) return MATGB_ERR_NOMEM;
      elem_t *Z = V + (size_t)(kdim + 1) * n;
      elem_t *D = Z + (size_t)kdim * n;
      MGB_CUDA(cudaMemcpyAsync(V, R, (size_t)n * sizeof(elem_t),
                               cudaMemcpyDeviceToDevice, st));
      double xn_known = 0;
      while (it < maxit) {
        int inner = 0;
        double est = 0;
        const int mcap = (int)std::min<int64_t>(kdim, maxit - it);
        // first cycle: ten orders of reduction; later ones: the absolute
        // residual that meets the backward-error target with room to spare
        const double atol =
            refinements == 0 ? 0.0 : 0.25 * tol * (anorm * xn_known + bn[0]);
        // with 16-bit factors and a fallback available, a first cycle that
        // has not gained three orders of magnitude in 24 steps gives up
        int stalled = 0;
        const bool may_abort = lp >= 0 && o.fp32_fallback && refinements == 0;
        const KrylovTarget tg{tol, anorm, bn[0]};
        MGB_TRY(fgmres_cycle(spd, n, A, lda, W, piv + n, V, Z, RF, mcap, 1e-10,
                             atol, may_abort ? 24 : 1 << 30, 1e-3,
                             refinements == 0 ? &tg : nullptr, D, &inner, &est,
                             &stalled));
        it += inner;
        ksteps += inner;
        if (stalled) break;
        MGB_CUDA(cudaMemsetAsync(dn, 0, sizeof(unsigned long long), st));
        add_vec_kernel<elem_t><<<grid_cap(n), 256, 0, st>>>(n, X, D, dn);
        MGB_LAUNCHED("add_vec");
        refinements++;
        // true residual in the element type
        MGB_CUDA(cudaMemcpyAsync(V, B, (size_t)n * sizeof(elem_t),
                                 cudaMemcpyDeviceToDevice, st));
        MGB_TRY(gemv_t<elem_t>(n, n, elem_t(-1), A, lda, X, elem_t(1), V));
        MGB_CUDA(cudaMemsetAsync(rs, 0, 2 * sizeof(unsigned long long), st));
        col_amax2_kernel<elem_t><<<cg, 256, 0, st>>>(n, V, n, X, ldx, rs);
        MGB_LAUNCHED("col_amax");
        MGB_TRY(fetch(rs, hv.data(), 3));  // rs[0..1], then dn[0]
        rn = hv[0];
        xn = hv[1];
        xn_known = xn;
        fwd = xn > 0 ? hv[2] / xn : (hv[2] == 0 ? 0.0 : INFINITY);
        const double den = anorm * xn + bn[0];
        eta = (den > 0) ? rn / den : (rn == 0 ? 0.0 : INFINITY);
        if (rn != rn || den != den) eta = NAN;
        if (eta <= tol) {
          converged = 1;
          break;
        }
        if (!(eta < 0.9 * prev)) break;  // stagnation or divergence
        prev = eta;
      }
      // Forward-error estimate: the correction the factors give for the final
      // residual, |M^-1 r|_inf / |x|_inf (the error e = A^-1 r, with M the
      // low-precision factors standing in for A).  The last FGMRES
      // correction is no estimate here: the first cycle starts from x = 0.
      // One preconditioner application, a fraction of a percent of a solve.
      if (refinements > 0 && xn > 0 && rn > 0 && rn == rn) {
        unsigned long long *fe = red + 2;  // free during refinement
        MGB_CUDA(cudaMemsetAsync(fe, 0, 2 * sizeof(unsigned long long), st));
        scale_to_float_kernel<elem_t><<<cg, 256, 0, st>>>(n, V, n, rs, RF);
        MGB_LAUNCHED("scale_to_float");
        MGB_TRY(precond_solve(spd, n, W, piv + n, RF, DF));
        col_amax2_kernel<float><<<cg, 256, 0, st>>>(n, DF, n, DF, n, fe);
        MGB_LAUNCHED("col_amax");
        MGB_TRY(fetch(fe, hv.data(), 1));
        fwd = hv[0] * rn / xn;
      } else if (rn == 0 && refinements > 0) {
        fwd = 0;
      }
    }
    // FP64 residuals of many right-hand sides on the tensor cores (digit
    // slices of A made once per solve); see resid64.cu
    bool rz = false;
#ifdef MAT_DOUBLE_PRECISION
    if (!use_krylov && nrhs > 1 && n >= kResid64MinN && g_resid64_on) {
      MGB_TRY(resid64_prepare(n, A, lda));
      rz = true;
    }
#endif
    while (!use_krylov && it < maxit) {
      // correction D = (LU)^{-1} R in FP32, column-scaled (first pass: plain)
      MGB_CUDA(cudaMemsetAsync(rs, 0, (size_t)2 * nrhs * sizeof(unsigned long long), st));
      col_amax2_kernel<elem_t><<<cg, 256, 0, st>>>(n, R, n, R, n, rs);
      MGB_LAUNCHED("col_amax");
      scale_to_float_kernel<elem_t><<<cg, 256, 0, st>>>(n, R, n, rs, RF);
      MGB_LAUNCHED("scale_to_float");
      if (spd) {
        MGB_CUDA(cudaMemcpyAsync(DF, RF, (size_t)n * nrhs * sizeof(float),
                                 cudaMemcpyDeviceToDevice, st));
        MGB_TRY(potrs_t<float>(n, nrhs, W, n, DF, n, nullptr));
      } else {
        MGB_TRY(getrs_t<float>(n, nrhs, W, n, piv + n, RF, n, DF, n));
      }
      MGB_CUDA(cudaMemsetAsync(dn, 0, (size_t)nrhs * sizeof(unsigned long long), st));
      update_x_kernel<elem_t><<<cg, 256, 0, st>>>(n, X, ldx, DF, rs, dn);
      MGB_LAUNCHED("update_x");
      it++;
      refinements++;
      // residual R = B - A X in the refinement precision
      copy_cols_kernel<elem_t><<<gnn, 256, 0, st>>>(n, nrhs, B, ldb, R, n);
      MGB_LAUNCHED("copy_cols");
      if (nrhs == 1 && ldx >= n)
        MGB_TRY(gemv_t<elem_t>(n, n, elem_t(-1), A, lda, X, elem_t(1), R));
#ifdef MAT_DOUBLE_PRECISION
      else if (rz)
        MGB_TRY(resid64(n, nrhs, A, X, ldx, R, n));
#endif
      else
        MGB_TRY(gemm_skip_t<elem_t>(false, false, n, nrhs, n, elem_t(-1), A,
                                    lda, X, ldx, elem_t(1), R, n, 0, nullptr));
      MGB_CUDA(cudaMemsetAsync(rs, 0, (size_t)2 * nrhs * sizeof(unsigned long long), st));
      col_amax2_kernel<elem_t><<<cg, 256, 0, st>>>(n, R, n, X, ldx, rs);
      MGB_LAUNCHED("col_amax");
      MGB_TRY(fetch(rs, hv.data(), 3 * (int)nrhs));  // rs, then dn
      eta = 0;
      rn = 0;
      xn = 0;
      fwd = 0;
      for (int64_t c = 0; c < nrhs; c++) {
        const double r = hv[2 * c], xv = hv[2 * c + 1];
        const double dv = hv[2 * nrhs + c];
        const double f = xv > 0 ? dv / xv : (dv == 0 ? 0.0 : INFINITY);
        if (!(f <= fwd)) fwd = f;
        const double den = anorm * xv + bn[c];
        double e = (den > 0) ? r / den : (r == 0 ? 0.0 : INFINITY);
        if (r != r || den != den) e = NAN;
        if (!(e <= eta)) eta = e;  // NaN-propagating max
        if (!(r <= rn)) rn = r;
        if (!(xv <= xn)) xn = xv;
      }
      if (eta <= tol) {
        converged = 1;
        break;
      }
      if (!(eta < 0.5 * prev)) break;  // stagnation or divergence
      prev = eta;
    }
    // low-precision factors too coarse for this matrix (kappa * u_low >~ 1):
    // refactor once with FP32 trailing updates and refine again
    if (converged || lp < 0 || !o.fp32_fallback || it >= maxit) break;
    lp = -1;
  }
  MGB_CUDA(cudaEventRecord(g_ir.e[2], st));
  MGB_CUDA(cudaEventSynchronize(g_ir.e[2]));
  if (tc_error_flag(1))
    return set_error(MATGB_ERR_TIMEOUT, "tensor-core update gave up waiting");
  if (lu_wait_error(1))
    return set_error(MATGB_ERR_TIMEOUT, "LU panel exchange gave up waiting");
  MGB_TRY(trsv_status());
  MGB_TRY(trsm_flag_status());
  if (rep) {
    float t = 0;
    cudaEventElapsedTime(&t, g_ir.e[1], g_ir.e[2]);
    double bmax = 0;
    for (double v : bn) bmax = v > bmax ? v : bmax;
    rep->iterations = it;
    rep->converged = converged;
    rep->backward_error = eta;
    rep->residual_inf = rn;
    rep->x_inf = xn;
    rep->a_inf = anorm;
    rep->b_inf = bmax;
    rep->tol = tol;
    rep->ms_factor = ms_factor;
    rep->ms_refine = t;
    rep->lp_format = lp;
    rep->refinements = refinements;
    rep->krylov_steps = ksteps;
    rep->forward_error_est = fwd;
  }
  return 0;
}

int gesv_ir(int64_t n, const elem_t *A, int64_t lda, const elem_t *b,
            elem_t *x, const MatIROpts &o, MatIRReport *rep,
            const elem_t *hA = nullptr) {
  return solve_ir(false, n, 1, A, lda, b, n, x, n, o, rep, nullptr, hA);
}

}  // namespace mgb

using namespace mgb;

extern "C" {

void matgb_ir_default_opts(MatIROpts *o) {
  o->lp_format = 2;
  o->max_iter = 100;
  o->tol = 0.0;
  o->fp32_fallback = 1;
  o->krylov = 1;
  o->krylov_dim = 50;
}

int matgb_resid64_mode(int on) {
  mgb::g_resid64_on = on ? 1 : 0;
  return 0;
}

int matgb_resid64_dev(size_t n, size_t nrhs, const mat_elem_t *A, size_t lda,
                      const mat_elem_t *X, size_t ldx, mat_elem_t *R, size_t ldr) {
#ifdef MAT_DOUBLE_PRECISION
  if (lda < n || ldx < n || ldr < n) return set_error(MATGB_ERR_ARG, "resid64: leading dimension");
  if (n == 0 || nrhs == 0) return 0;
  MGB_TRY(resid64_prepare((int64_t)n, A, (int64_t)lda));
  return resid64((int64_t)n, (int64_t)nrhs, A, X, (int64_t)ldx, R, (int64_t)ldr);
#else
  (void)n; (void)nrhs; (void)A; (void)lda; (void)X; (void)ldx; (void)R; (void)ldr;
  return set_error(MATGB_ERR_ARG, "resid64: double precision only");
#endif
}

int matgb_getrf_lp_dev(size_t n, float *A, size_t lda, int32_t *ipiv,
                       int32_t *perm, int lp_format) {
  if (lda < n) return set_error(MATGB_ERR_ARG, "getrf_lp: lda < n");
  if (lp_format < -1 || lp_format > 3)
    return set_error(MATGB_ERR_ARG, "getrf_lp: lp_format");
  return getrf_t<float>((int64_t)n, A, (int64_t)lda, ipiv, perm, 0.f,
                        lp_format);
}

int matgb_gesv_ir_dev(size_t n, const mat_elem_t *A, size_t lda,
                      const mat_elem_t *b, mat_elem_t *x,
                      const MatIROpts *opts, MatIRReport *rep) {
  if (lda < n) return set_error(MATGB_ERR_ARG, "gesv_ir: lda < n");
  MatIROpts o;
  matgb_ir_default_opts(&o);
  if (opts) o = *opts;
  return gesv_ir((int64_t)n, A, (int64_t)lda, b, x, o, rep);
}

int matgb_gesv_ir_multi_dev(size_t n, size_t nrhs, const mat_elem_t *A,
                            size_t lda, const mat_elem_t *B, size_t ldb,
                            mat_elem_t *X, size_t ldx, const MatIROpts *opts,
                            MatIRReport *rep) {
  if (lda < n || ldb < n || ldx < n)
    return set_error(MATGB_ERR_ARG, "gesv_ir: leading dimension too small");
  MatIROpts o;
  matgb_ir_default_opts(&o);
  if (opts) o = *opts;
  return solve_ir(false, (int64_t)n, (int64_t)nrhs, A, (int64_t)lda, B,
                  (int64_t)ldb, X, (int64_t)ldx, o, rep, nullptr);
}

int matgb_posv_ir_dev(size_t n, size_t nrhs, const mat_elem_t *A, size_t lda,
                      const mat_elem_t *B, size_t ldb, mat_elem_t *X,
                      size_t ldx, const MatIROpts *opts, MatIRReport *rep) {
  if (lda < n || ldb < n || ldx < n)
    return set_error(MATGB_ERR_ARG, "posv_ir: leading dimension too small");
  MatIROpts o;
  matgb_ir_default_opts(&o);
  if (opts) o = *opts;
  int not_spd = 0;
  MGB_TRY(solve_ir(true, (int64_t)n, (int64_t)nrhs, A, (int64_t)lda, B,
                   (int64_t)ldb, X, (int64_t)ldx, o, rep, &not_spd));
  return not_spd ? -1 : 0;
}

int mat_solve_spd_ir(Vec *x, const Mat *A, const Vec *b, const MatIROpts *opts,
                     MatIRReport *rep) {
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(x);
  MAT_ASSERT_MAT(b);
  MAT_ASSERT_SQUARE(A);
  MAT_ASSERT(b->rows == A->rows && x->rows == A->cols);
  MAT_ASSERT(x->cols == b->cols);
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows, nr = b->cols;
  cudaStream_t st = ctx()->stream;
  elem_t *dA = (elem_t *)ws(WS_A, (size_t)n * n * sizeof(elem_t));
  elem_t *db = (elem_t *)ws(WS_B, (size_t)n * nr * sizeof(elem_t));
  elem_t *dx = (elem_t *)ws(WS_X, (size_t)n * nr * sizeof(elem_t));
  if (!dA || !db || !dx) return MATGB_ERR_NOMEM;
  MGB_CUDA(cudaMemcpyAsync(dA, A->data, (size_t)n * n * sizeof(elem_t),
                           cudaMemcpyHostToDevice, st));
  MGB_CUDA(cudaMemcpyAsync(db, b->data, (size_t)n * nr * sizeof(elem_t),
                           cudaMemcpyHostToDevice, st));
  MatIROpts o;
  matgb_ir_default_opts(&o);
  if (opts) o = *opts;
  int not_spd = 0;
  MGB_TRY(solve_ir(true, n, nr, dA, n, db, n, dx, n, o, rep, &not_spd));
  if (not_spd) return -1;
  MGB_CUDA(cudaMemcpyAsync(x->data, dx, (size_t)n * nr * sizeof(elem_t),
                           cudaMemcpyDeviceToHost, st));
  MGB_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int mat_solve_ir(Vec *x, const Mat *A, const Vec *b, const MatIROpts *opts,
                 MatIRReport *rep) {
  MAT_ASSERT_MAT(A);
  MAT_ASSERT_MAT(x);
  MAT_ASSERT_MAT(b);
  MAT_ASSERT_SQUARE(A);
  MAT_ASSERT(b->rows == A->rows && x->rows == A->cols);
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  const int64_t n = A->rows;
  cudaStream_t st = ctx()->stream;
  elem_t *dA = (elem_t *)ws(WS_A, (size_t)n * n * sizeof(elem_t));
  elem_t *db = (elem_t *)ws(WS_B, (size_t)n * sizeof(elem_t));
  elem_t *dx = (elem_t *)ws(WS_X, (size_t)n * sizeof(elem_t));
  if (!dA || !db || !dx) return MATGB_ERR_NOMEM;
  MGB_CUDA(cudaMemcpyAsync(db, b->data, (size_t)n * sizeof(elem_t),
                           cudaMemcpyHostToDevice, st));
  MatIROpts o;
  matgb_ir_default_opts(&o);
  if (opts) o = *opts;
  // A is copied in column chunks while the factorisation runs
  MGB_TRY(gesv_ir(n, dA, n, db, dx, o, rep, A->data));
  MGB_CUDA(cudaMemcpyAsync(x->data, dx, (size_t)n * sizeof(elem_t),
                           cudaMemcpyDeviceToHost, st));
  MGB_CUDA(cudaStreamSynchronize(st));
  return 0;
}

}  // extern "C"
