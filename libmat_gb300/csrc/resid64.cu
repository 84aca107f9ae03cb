// FP64 residual R -= A X for a block of right-hand sides, on the tensor
// cores.
//
// GB300 runs FP64 at ~1.25 TFLOP/s, so the refinement's residual for 64
// right-hand sides (2 n^2 * 64 FLOP) would cost more than the whole mixed
// factorisation.  It is formed here from exact FP16 products instead, by
// the slicing scheme of Ozaki, Ogita and Oishi (2012):
//   - every row of A and every column of X is scaled by a power of two (its
//     largest magnitude below 1);
//   - each scaled value is cut into 8 signed 7-bit digits, every digit an
//     integer held exactly in FP16;
//   - a product of two digits is below 2^14, so a sum of 1024 of them stays
//     below 2^24: the tensor-core GEMM of a digit pair over a 1024-term
//     chunk of the inner dimension is exact in FP32;
//   - the chunk results are scaled by their powers of two and accumulated
//     in FP64.
// Digit pairs weighted below 2^-63 are left out.  A value is represented to
// 2^-56 of its row's (column's) largest magnitude, so the residual's error
// is below about n * 2^-55 * max|A_i.| * max|x| per row -- the bound of an
// FP64 GEMM.  Non-finite entries make all their digits NaN, which carries
// into R as an FP64 GEMM would carry it.
#include <cuda_fp16.h>

#include "internal.cuh"

namespace mgb {

constexpr int kRzSlices = 8;   // digits per value
constexpr int kRzBits = 7;     // bits per digit (|digit| <= 127)
constexpr int kRzK = 1024;     // inner-dimension terms per exact FP32 sum
constexpr int kRzN = 64;       // right-hand sides per pass

// Scale exponents: e with max |v| < 2^e (frexp's); rows or columns with no
// nonzero keep a sentinel below any exponent (all their digits are zero),
// and a non-finite entry gives the NaN marker INT_MAX.
constexpr int kRzNaN = INT_MAX;
constexpr int kRzNone = -2000000000;  // below every frexp exponent (>= -1074)
__device__ __forceinline__ int rz_exp(double mx) {
  if (!(mx <= 1.7976931348623157e308)) return kRzNaN;  // inf or NaN
  if (!(mx > 0)) return kRzNone;
  int e = 0;
  frexp(mx, &e);
  return e;
}

// Row maxima of |A| as exponents, by 32 x 32 tiles (coalesced down the
// columns): each tile's row maxima are merged with atomicMax, the exponent
// growing with the magnitude.  e is preset to a value at or below kRzNone.
__global__ void __launch_bounds__(256)
    rz_row_exp_kernel(int64_t n, const double *__restrict__ A, int64_t lda,
                      int *__restrict__ e) {
  // magnitudes compare as their bit patterns (NaN and inf above every
  // finite value), so the maxima need no FP64 arithmetic
  __shared__ unsigned long long t[8][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 rows x 8 column groups
  const int64_t i = (int64_t)blockIdx.y * 32 + tx, j0 = (int64_t)blockIdx.x * 32;
  unsigned long long mx = 0;
  if (i < n)
    for (int64_t j = j0 + ty; j < j0 + 32 && j < n; j += 8) {
      const unsigned long long b = __double_as_longlong(A[i + j * lda]) & 0x7fffffffffffffffull;
      mx = b > mx ? b : mx;
    }
  t[ty][tx] = mx;
  __syncthreads();
  if (ty == 0 && i < n) {
    unsigned long long m = t[0][tx];
    for (int g = 1; g < 8; g++) m = t[g][tx] > m ? t[g][tx] : m;
    const int ex = rz_exp(__longlong_as_double((long long)m));
    if (ex != kRzNone) atomicMax(&e[i], ex);
  }
}

// Column maxima of |X| as exponents: one block per column.
__global__ void rz_col_exp_kernel(int64_t n, const double *__restrict__ X, int64_t ldx,
                                  int *__restrict__ f) {
  __shared__ unsigned long long smx[8];
  const int k = blockIdx.x, tid = threadIdx.x;
  unsigned long long mx = 0;
  for (int64_t j = tid; j < n; j += blockDim.x) {
    const unsigned long long b =
        __double_as_longlong(X[j + (int64_t)k * ldx]) & 0x7fffffffffffffffull;
    mx = b > mx ? b : mx;
  }
  for (int off = 16; off; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, mx, off);
    mx = o > mx ? o : mx;
  }
  if ((tid & 31) == 0) smx[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) mx = smx[w] > mx ? smx[w] : mx;
    f[k] = rz_exp(__longlong_as_double((long long)mx));
  }
}

// The digits of v * 2^-e (|v * 2^-e| < 1): digit l is the integer part of
// the value scaled by 2^(7(l+1)) less 2^7 times digit l-1, i.e. bits
// 55-7l .. 49-7l of the 56-bit fraction floor(|v| 2^(56-e)), with v's sign.
// Integer operations on v's bit pattern (GB300's FP64 rate is low); the
// same digits as truncating in exact FP64 arithmetic.
__device__ __forceinline__ void rz_digits(double v, int e, uint16_t (&d)[kRzSlices]) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  const int ex = (int)((bits >> 52) & 0x7ff);
  if (e == kRzNaN || ex == 0x7ff) {
#pragma unroll
    for (int l = 0; l < kRzSlices; l++) d[l] = 0x7e00u;  // FP16 NaN
    return;
  }
  unsigned long long frac = 0;
  if (e > kRzNone) {
    const unsigned long long mant =
        (bits & 0x000fffffffffffffull) | (ex ? 0x0010000000000000ull : 0ull);
    // |v| = mant * 2^(max(ex,1) - 1075); frac = |v| * 2^(56 - e), < 2^56
    const int sh = (ex ? ex : 1) - 1075 + 56 - e;
    frac = sh >= 0 ? (sh < 11 ? mant << sh : 0ull) : (-sh < 64 ? mant >> -sh : 0ull);
  }
  const bool neg = (bits >> 63) != 0;
#pragma unroll
  for (int l = 0; l < kRzSlices; l++) {
    const int dig = (int)((frac >> (kRzBits * (kRzSlices - 1 - l))) & 127u);
    d[l] = __half_as_ushort(__int2half_rn(neg ? -dig : dig));
  }
}

// A (column-major, n x n) to its digit slices, row-major (K contiguous, the
// tensor-core kernel's A operand): slice l at S + l * sstride, row i at
// i * ld.  A 32 x 32 tile goes through shared memory so both the reads (down
// columns) and the writes (along rows) are coalesced; columns n..ld-1 are
// zero.
__global__ void __launch_bounds__(256)
    rz_slice_a_kernel(int64_t n, const double *__restrict__ A, int64_t lda,
                      const int *__restrict__ e, uint16_t *__restrict__ S, int64_t ld,
                      int64_t sstride) {
  __shared__ double t[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int64_t i0 = (int64_t)blockIdx.y * 32, j0 = (int64_t)blockIdx.x * 32;
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + tx, j = j0 + r;
    t[r][tx] = (i < n && j < n) ? A[i + j * lda] : 0.0;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + r, j = j0 + tx;
    if (i >= n || j >= ld) continue;
    uint16_t d[kRzSlices];
    rz_digits(t[tx][r], j < n ? e[i] : kRzNone, d);
#pragma unroll
    for (int l = 0; l < kRzSlices; l++) S[l * sstride + i * ld + j] = d[l];
  }
}

// X (column-major, n x nr, nr <= 64) to its digit slices as the B operand:
// row l*64 + k holds digit l of column k (K contiguous); rows for k >= nr
// and columns n..ld-1 are zero.
__global__ void rz_slice_x_kernel(int64_t n, int nr, const double *__restrict__ X,
                                  int64_t ldx, const int *__restrict__ f,
                                  uint16_t *__restrict__ S, int64_t ld) {
  const int k = blockIdx.y;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < ld;
       j += (int64_t)gridDim.x * blockDim.x) {
    uint16_t d[kRzSlices];
    if (k < nr && j < n) {
      rz_digits(X[j + (int64_t)k * ldx], f[k], d);
    } else {
#pragma unroll
      for (int l = 0; l < kRzSlices; l++) d[l] = 0;
    }
#pragma unroll
    for (int l = 0; l < kRzSlices; l++) S[((int64_t)l * kRzN + k) * ld + j] = d[l];
  }
}

// R(i, k) -= 2^(e_i + f_k) * sum over digit pairs (l, m), l + m <= 7, of
// 2^(-7(l+m+2)) * C_l(i, m*64 + k): C_l is the exact FP32 product of A's
// digit l with X's digits 0..7-l over one chunk of the inner dimension.
__global__ void rz_accum_kernel(int64_t n, int nr, const float *__restrict__ C,
                                int64_t ldc, const int64_t *__restrict__ coff,
                                const int *__restrict__ e, const int *__restrict__ f,
                                double *__restrict__ R, int64_t ldr) {
  const int k = blockIdx.y;
  if (k >= nr) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    // products of equal weight (l + m = s) summed exactly as integers (each
    // below 2^24, at most 8 of them: below 2^27), then one FP64 term per
    // weight
    int is[kRzSlices];
#pragma unroll
    for (int w = 0; w < kRzSlices; w++) is[w] = 0;
    bool nan = false;
#pragma unroll
    for (int l = 0; l < kRzSlices; l++) {
      const float *Cl = C + coff[l];
#pragma unroll
      for (int m = 0; m + l < kRzSlices; m++) {
        const float c = Cl[i + (int64_t)(m * kRzN + k) * ldc];
        nan = nan || c != c;
        is[l + m] += (int)c;
      }
    }
    // weights 2^(-7(w+2)) are exact doubles: a multiply, not ldexp (FP64
    // runs at a low rate on this part)
    double acc = 0;
#pragma unroll
    for (int w = kRzSlices - 1; w >= 0; w--)
      acc = fma((double)is[w], __longlong_as_double((long long)(1023 - kRzBits * (w + 2)) << 52), acc);
    if (nan) acc = NAN;
    const int ei = e[i], fk = f[k];
    double v;
    if (ei == kRzNaN || fk == kRzNaN)
      v = NAN;
    else if (ei <= kRzNone || fk <= kRzNone)
      v = acc;  // zero: every digit of the row (column) is zero
    else {
      const int E = ei + fk;  // 2^E exactly, by its bit pattern where normal
      v = (E >= -1022 && E <= 1023) ? acc * __longlong_as_double((long long)(E + 1023) << 52)
                                    : ldexp(acc, E);
    }
    R[i + (int64_t)k * ldr] -= v;
  }
}

// Sliced A, kept for the residuals of one solve.
struct RzState {
  const double *A = nullptr;
  int64_t n = 0, lda = 0, ld = 0;
  uint16_t *SA = nullptr;
};
static RzState g_rz;

int resid64_prepare(int64_t n, const double *A, int64_t lda) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  const int64_t ld = (n + kRzK - 1) / kRzK * kRzK;
  const int64_t sstride = n * ld;
  uint16_t *SA = (uint16_t *)ws(WS_RZA, (size_t)kRzSlices * sstride * sizeof(uint16_t));
  int *e = (int *)ws(WS_RZE, (size_t)(n + kRzN) * sizeof(int));
  if (!SA || !e) return MATGB_ERR_NOMEM;
  cudaStream_t st = cx->stream;
  {
    KtScope kt("resid64_slice_a", 0.0, (double)n * n * 8 + (double)kRzSlices * sstride * 2);
    MGB_CUDA(cudaMemsetAsync(e, 0x88, (size_t)n * sizeof(int), st));  // below kRzNone
    dim3 ge((unsigned)((n + 31) / 32), (unsigned)((n + 31) / 32));
    rz_row_exp_kernel<<<ge, 256, 0, st>>>(n, A, lda, e);
    MGB_LAUNCHED("rz_row_exp");
    dim3 g((unsigned)((ld + 31) / 32), (unsigned)((n + 31) / 32));
    rz_slice_a_kernel<<<g, 256, 0, st>>>(n, A, lda, e, SA, ld, sstride);
    MGB_LAUNCHED("rz_slice_a");
  }
  g_rz.A = A;
  g_rz.n = n;
  g_rz.lda = lda;
  g_rz.ld = ld;
  g_rz.SA = SA;
  return 0;
}

int resid64(int64_t n, int64_t nrhs, const double *A, const double *X, int64_t ldx,
            double *R, int64_t ldr) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (g_rz.A != A || g_rz.n != n || !g_rz.SA)
    return set_error(MATGB_ERR_ARG, "resid64: A not prepared");
  const int64_t ld = g_rz.ld, sstride = n * ld;
  int *e = (int *)ws(WS_RZE, (size_t)(n + kRzN) * sizeof(int));
  int *f = e + n;
  uint16_t *SX = (uint16_t *)ws(WS_RZB, (size_t)kRzSlices * kRzN * ld * sizeof(uint16_t));
  // C_l: n x 64(8-l) FP32, one after another, plus their offsets
  int64_t coffs[kRzSlices], tot = 0;
  for (int l = 0; l < kRzSlices; l++) {
    coffs[l] = tot;
    tot += n * (int64_t)kRzN * (kRzSlices - l);
  }
  float *C = (float *)ws(WS_RZC, (size_t)tot * sizeof(float) + 256);
  if (!SX || !C) return MATGB_ERR_NOMEM;
  int64_t *doff = (int64_t *)((char *)C + (size_t)tot * sizeof(float));
  cudaStream_t st = cx->stream;
  MGB_CUDA(cudaMemcpyAsync(doff, coffs, sizeof(coffs), cudaMemcpyHostToDevice, st));
  for (int64_t c0 = 0; c0 < nrhs; c0 += kRzN) {
    const int nr = (int)((nrhs - c0) < kRzN ? (nrhs - c0) : kRzN);
    const double *Xc = X + c0 * ldx;
    double *Rc = R + c0 * ldr;
    {
      KtScope kt("resid64_slice_x", 0.0, (double)n * nr * 8 + (double)kRzSlices * kRzN * ld * 2);
      rz_col_exp_kernel<<<nr, 256, 0, st>>>(n, Xc, ldx, f);
      MGB_LAUNCHED("rz_col_exp");
      dim3 gx((unsigned)((ld + 255) / 256 < 256 ? (ld + 255) / 256 : 256), kRzN);
      rz_slice_x_kernel<<<gx, 256, 0, st>>>(n, nr, Xc, ldx, f, SX, ld);
      MGB_LAUNCHED("rz_slice_x");
    }
    for (int64_t k0 = 0; k0 < ld; k0 += kRzK) {
      for (int l = 0; l < kRzSlices; l++)
        MGB_TRY(tc_gemm(0, n, (int64_t)kRzN * (kRzSlices - l), kRzK,
                        g_rz.SA + l * sstride + k0, ld, SX + k0, ld, 1.f, nullptr, 0.f,
                        C + coffs[l], n, 0, nullptr));
      KtScope kt("resid64_accum", 0.0, (double)tot * 4 + 16.0 * n * nr);
      dim3 ga((unsigned)((n + 255) / 256 < 512 ? (n + 255) / 256 : 512), (unsigned)nr);
      rz_accum_kernel<<<ga, 256, 0, st>>>(n, nr, C, n, doff, e, f, Rc, ldr);
      MGB_LAUNCHED("rz_accum");
    }
  }
  return 0;
}

}  // namespace mgb
