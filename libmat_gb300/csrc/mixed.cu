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

#include "internal.cuh"

namespace mgb {

// ---- packing the trailing-update operands -------------------------------------
template <int BF16>
__device__ __forceinline__ uint16_t to16(float v) {
  if (BF16) return __bfloat16_as_ushort(__float2bfloat16_rn(v));
  return __half_as_ushort(__float2half_rn(v));
}

// out[i*Kp + k] = A[i + k*lda] for i < m, k < nb (zero for nb <= k < Kp):
// L21 (column-major, M-contiguous) to a K-contiguous 16-bit operand.
template <int BF16>
__global__ void pack_l21_kernel(const float *__restrict__ A, int64_t lda,
                                int64_t m, int nb, int Kp,
                                uint16_t *__restrict__ out) {
  __shared__ float t[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int64_t i0 = (int64_t)blockIdx.x * 32;
  const int k0 = blockIdx.y * 32;
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + tx;
    const int k = k0 + r;
    t[r][tx] = (i < m && k < nb) ? A[i + (int64_t)k * lda] : 0.f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + r;
    if (i < m) out[i * Kp + k0 + tx] = to16<BF16>(t[tx][r]);
  }
}

// FP16 scale of U12: s = 2^(14 - ceil(log2 max|U12|)), so the largest entry
// maps to at most 2^14; scale[0] = s, scale[1] = 1/s (both exact).
__global__ void u12_amax_kernel(const float *__restrict__ A, int64_t lda,
                                int nb, int64_t ncols,
                                unsigned *__restrict__ amax_bits) {
  float m = 0.f;
  const int64_t tot = (int64_t)nb * ncols;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const float v = fabsf(A[(e % nb) + (e / nb) * lda]);
    if (v > m) m = v;  // NaN is ignored here; it propagates through the GEMM
  }
  for (int off = 16; off; off >>= 1) m = fmaxf(m, __shfl_xor_sync(~0u, m, off));
  if ((threadIdx.x & 31) == 0) atomicMax(amax_bits, __float_as_uint(m));
}

__device__ __forceinline__ float fp16_scale(unsigned amax_bits) {
  const float a = __uint_as_float(amax_bits);
  if (!(a > 0.f) || isinf(a)) return 1.f;
  int e;
  frexpf(a, &e);  // a = f * 2^e, f in [0.5, 1)
  return ldexpf(1.f, 14 - e);
}

// out[j*Kp + k] = s * A[k + j*lda] (k < nb), 0 for nb <= k < Kp.
template <int BF16>
__global__ void pack_u12_kernel(const float *__restrict__ A, int64_t lda,
                                int nb, int Kp, int64_t ncols,
                                const unsigned *__restrict__ amax_bits,
                                float *__restrict__ scale,
                                uint16_t *__restrict__ out) {
  const float s = (!BF16 && amax_bits) ? fp16_scale(*amax_bits) : 1.f;
  if (blockIdx.x == 0 && threadIdx.x == 0 && scale) {
    scale[0] = s;
    scale[1] = 1.f / s;
  }
  const int64_t tot = (int64_t)Kp * ncols;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % Kp);
    const int64_t j = e / Kp;
    out[e] = to16<BF16>(k < nb ? s * A[k + j * lda] : 0.f);
  }
}

static unsigned grid_cap(int64_t tot, int per = 256) {
  int64_t b = (tot + per - 1) / per;
  int64_t cap = (int64_t)ctx()->sms * 16;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

int lp_trailing_update(int64_t n, float *A, int64_t lda, int64_t kb,
                       int64_t ke, int64_t c0, int64_t c1, int lp, bool pack) {
  const int nb = (int)(ke - kb);
  const int Kp = (nb + 63) / 64 * 64;
  const int64_t m = n - ke, ncols = n - ke;
  uint16_t *A16 = (uint16_t *)ws(WS_T0, (size_t)m * Kp * 2);
  uint16_t *B16 = (uint16_t *)ws(WS_T1, (size_t)ncols * Kp * 2);
  float *sc = (float *)ws(WS_T2, 64);
  if (!A16 || !B16 || !sc) return MATGB_ERR_NOMEM;
  unsigned *amax = (unsigned *)(sc + 4);
  cudaStream_t st = ctx()->stream;
  if (pack) {
    KtScope kt("lp_pack", 0.0, 6.0 * (m + ncols) * nb);
    dim3 g((unsigned)((m + 31) / 32), (unsigned)(Kp / 32));
    if (lp == 1)
      pack_l21_kernel<1><<<g, 256, 0, st>>>(A + ke + kb * lda, lda, m, nb, Kp, A16);
    else
      pack_l21_kernel<0><<<g, 256, 0, st>>>(A + ke + kb * lda, lda, m, nb, Kp, A16);
    MGB_LAUNCHED("pack_l21");
    const float *U12 = A + kb + ke * lda;
    if (lp == 0) {
      MGB_CUDA(cudaMemsetAsync(amax, 0, sizeof(unsigned), st));
      u12_amax_kernel<<<grid_cap((int64_t)nb * ncols), 256, 0, st>>>(
          U12, lda, nb, ncols, amax);
      MGB_LAUNCHED("u12_amax");
      pack_u12_kernel<0><<<grid_cap((int64_t)Kp * ncols), 256, 0, st>>>(
          U12, lda, nb, Kp, ncols, amax, sc, B16);
    } else {
      pack_u12_kernel<1><<<grid_cap((int64_t)Kp * ncols), 256, 0, st>>>(
          U12, lda, nb, Kp, ncols, nullptr, sc, B16);
    }
    MGB_LAUNCHED("pack_u12");
  }
  return tc_gemm(lp == 1, m, c1 - c0, Kp, A16, Kp, B16 + (c0 - ke) * Kp, Kp,
                 -1.f, lp == 0 ? sc + 1 : nullptr, 1.f, A + ke + c0 * lda, lda);
}

// ---- refinement kernels ------------------------------------------------------------
template <typename S>
__global__ void to_float_kernel(int64_t rows, int64_t cols,
                                const S *__restrict__ A, int64_t lda,
                                float *__restrict__ W, int64_t ldw) {
  const int64_t tot = rows * cols;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < tot;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % rows, j = e / rows;
    W[i + j * ldw] = (float)A[i + j * lda];
  }
}

// max over rows of sum_j |A(i,j)| (|A|_inf), via the bit pattern of a
// non-negative double (monotone as an unsigned integer).
template <typename S>
__global__ void row_abs_sum_kernel(int64_t n, const S *__restrict__ A,
                                   int64_t lda,
                                   unsigned long long *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int64_t j = 0; j < n; j++) s += fabs((double)A[i + j * lda]);
  atomicMax(out, (unsigned long long)__double_as_longlong(s));
}

template <typename S>
__global__ void amax2_kernel(int64_t n, const S *__restrict__ x,
                             const S *__restrict__ y,
                             unsigned long long *__restrict__ out) {
  double mx = 0, my = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double a = fabs((double)x[i]), b = fabs((double)y[i]);
    mx = a > mx || a != a ? a : mx;
    my = b > my || b != b ? b : my;
  }
  for (int off = 16; off; off >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(~0u, mx, off));
    my = fmax(my, __shfl_xor_sync(~0u, my, off));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, (unsigned long long)__double_as_longlong(mx));
    atomicMax(out + 1, (unsigned long long)__double_as_longlong(my));
  }
}

// rf = r / rn in FP32 (rn read from the device, 1 when zero)
template <typename S>
__global__ void scale_to_float_kernel(int64_t n, const S *__restrict__ r,
                                      const unsigned long long *__restrict__ rn,
                                      float *__restrict__ rf) {
  double s = __longlong_as_double((long long)rn[0]);
  s = (s > 0 && s < INFINITY) ? 1.0 / s : 1.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    rf[i] = (float)((double)r[i] * s);
}

// x += rn * d
template <typename S>
__global__ void update_x_kernel(int64_t n, S *__restrict__ x,
                                const float *__restrict__ d,
                                const unsigned long long *__restrict__ rn) {
  double s = __longlong_as_double((long long)rn[0]);
  if (!(s > 0 && s < INFINITY)) s = 1.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = (S)((double)x[i] + s * (double)d[i]);
}

// Two reduced doubles (stored as their bit patterns) to the host.
static int fetch2(const unsigned long long *d, double v[2]) {
  unsigned long long h[2] = {0, 0};
  MGB_CUDA(cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost,
                           ctx()->stream));
  MGB_CUDA(cudaStreamSynchronize(ctx()->stream));
  memcpy(v, h, sizeof h);
  return 0;
}

struct IrEvents {
  cudaEvent_t e[3];
  bool ready = false;
};
static IrEvents g_ir;

// Solve A x = b (A n x n in the library type, column-major) with the
// mixed-precision factorisation and refinement.  x may start anywhere: it is
// overwritten.
int gesv_ir(int64_t n, const elem_t *A, int64_t lda, const elem_t *b,
            elem_t *x, const MatIROpts &o, MatIRReport *rep) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (n <= 0) return 0;
  if (o.lp_format != 0 && o.lp_format != 1)
    return set_error(MATGB_ERR_ARG, "lp_format must be 0 (FP16) or 1 (BF16)");
  if (!g_ir.ready) {
    for (auto &e : g_ir.e) MGB_CUDA(cudaEventCreate(&e));
    g_ir.ready = true;
  }
  cudaStream_t st = cx->stream;
  float *W = (float *)ws(WS_U, (size_t)n * n * sizeof(float));
  int32_t *piv = (int32_t *)ws(WS_PIV, (size_t)2 * n * sizeof(int32_t));
  elem_t *r = (elem_t *)ws(WS_V0, (size_t)n * sizeof(elem_t));
  float *rf = (float *)ws(WS_V1, (size_t)2 * n * sizeof(float));
  unsigned long long *red =
      (unsigned long long *)ws(WS_INFO, 8 * sizeof(unsigned long long));
  if (!W || !piv || !r || !rf || !red) return MATGB_ERR_NOMEM;
  float *df = rf + n;

  MGB_CUDA(cudaEventRecord(g_ir.e[0], st));
  to_float_kernel<elem_t><<<grid_cap(n * n), 256, 0, st>>>(n, n, A, lda, W, n);
  MGB_LAUNCHED("to_float");
  MGB_TRY(getrf_t<float>(n, W, n, piv, piv + n, 0.f, o.lp_format));
  MGB_CUDA(cudaEventRecord(g_ir.e[1], st));

  MGB_CUDA(cudaMemsetAsync(red, 0, 8 * sizeof(unsigned long long), st));
  row_abs_sum_kernel<elem_t><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(
      n, A, lda, red + 4);
  MGB_LAUNCHED("row_abs_sum");
  amax2_kernel<elem_t><<<grid_cap(n), 256, 0, st>>>(n, b, b, red + 2);
  MGB_LAUNCHED("amax");
  double nv[2], av[2];
  MGB_TRY(fetch2(red + 2, nv));
  MGB_TRY(fetch2(red + 4, av));
  const double anorm = av[0], bnorm = nv[0];
  const double eps = sizeof(elem_t) == 8 ? 1.1102230246251565e-16
                                         : 5.960464477539063e-08;
  const double tol = o.tol > 0 ? o.tol : (double)n * eps;
  const int maxit = o.max_iter > 0 ? o.max_iter : 30;

  MGB_CUDA(cudaMemsetAsync(x, 0, (size_t)n * sizeof(elem_t), st));
  MGB_CUDA(cudaMemcpyAsync(r, b, (size_t)n * sizeof(elem_t),
                           cudaMemcpyDeviceToDevice, st));
  double eta = INFINITY, rn = bnorm, xn = 0, prev = INFINITY;
  int it = 0, converged = 0;
  while (it < maxit) {
    // correction d = (LU)^{-1} r in FP32 (the first pass is the plain solve)
    MGB_CUDA(cudaMemsetAsync(red, 0, 2 * sizeof(unsigned long long), st));
    amax2_kernel<elem_t><<<grid_cap(n), 256, 0, st>>>(n, r, r, red);
    MGB_LAUNCHED("amax");
    scale_to_float_kernel<elem_t><<<grid_cap(n), 256, 0, st>>>(n, r, red, rf);
    MGB_LAUNCHED("scale_to_float");
    MGB_TRY(getrs_t<float>(n, 1, W, n, piv + n, rf, n, df, n));
    update_x_kernel<elem_t><<<grid_cap(n), 256, 0, st>>>(n, x, df, red);
    MGB_LAUNCHED("update_x");
    it++;
    // residual of the updated x in the refinement precision
    MGB_CUDA(cudaMemcpyAsync(r, b, (size_t)n * sizeof(elem_t),
                             cudaMemcpyDeviceToDevice, st));
    MGB_TRY(gemv_t<elem_t>(n, n, elem_t(-1), A, lda, x, elem_t(1), r));
    MGB_CUDA(cudaMemsetAsync(red, 0, 2 * sizeof(unsigned long long), st));
    amax2_kernel<elem_t><<<grid_cap(n), 256, 0, st>>>(n, r, x, red);
    MGB_LAUNCHED("amax");
    double v[2];
    MGB_TRY(fetch2(red, v));
    rn = v[0];
    xn = v[1];
    const double den = anorm * xn + bnorm;
    eta = den > 0 ? rn / den : (rn > 0 ? INFINITY : 0.0);
    if (eta <= tol) {
      converged = 1;
      break;
    }
    // stop when refinement stagnates or diverges
    if (!(eta < 0.5 * prev)) break;
    prev = eta;
  }
  MGB_CUDA(cudaEventRecord(g_ir.e[2], st));
  MGB_CUDA(cudaEventSynchronize(g_ir.e[2]));
  if (tc_error_flag(1))
    return set_error(MATGB_ERR_TIMEOUT, "tensor-core update gave up waiting");
  if (rep) {
    float f = 0, t = 0;
    cudaEventElapsedTime(&f, g_ir.e[0], g_ir.e[1]);
    cudaEventElapsedTime(&t, g_ir.e[1], g_ir.e[2]);
    rep->iterations = it;
    rep->converged = converged;
    rep->backward_error = eta;
    rep->residual_inf = rn;
    rep->x_inf = xn;
    rep->a_inf = anorm;
    rep->b_inf = bnorm;
    rep->tol = tol;
    rep->ms_factor = f;
    rep->ms_refine = t;
    rep->lp_format = o.lp_format;
  }
  return 0;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

void matgb_ir_default_opts(MatIROpts *o) {
  o->lp_format = 1;
  o->max_iter = 30;
  o->tol = 0.0;
}

int matgb_getrf_lp_dev(size_t n, float *A, size_t lda, int32_t *ipiv,
                       int32_t *perm, int lp_format) {
  if (lda < n) return set_error(MATGB_ERR_ARG, "getrf_lp: lda < n");
  if (lp_format < -1 || lp_format > 1)
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
  MGB_CUDA(cudaMemcpyAsync(dA, A->data, (size_t)n * n * sizeof(elem_t),
                           cudaMemcpyHostToDevice, st));
  MGB_CUDA(cudaMemcpyAsync(db, b->data, (size_t)n * sizeof(elem_t),
                           cudaMemcpyHostToDevice, st));
  MatIROpts o;
  matgb_ir_default_opts(&o);
  if (opts) o = *opts;
  MGB_TRY(gesv_ir(n, dA, n, db, dx, o, rep));
  MGB_CUDA(cudaMemcpyAsync(x->data, dx, (size_t)n * sizeof(elem_t),
                           cudaMemcpyDeviceToHost, st));
  MGB_CUDA(cudaStreamSynchronize(st));
  return 0;
}

}  // extern "C"
