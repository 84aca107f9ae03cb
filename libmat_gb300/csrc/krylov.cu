// Flexible GMRES for the correction equation of the mixed-precision solvers.
//
// Refinement with a low-precision factorisation converges only while
// kappa(A) * u_low < 1 (u_low = 2^-8 for BF16, 2^-11 for FP16 factors).  To
// keep the tensor-core factorisation for worse-conditioned systems the
// correction A d = r is solved by right-preconditioned flexible GMRES in the
// library's element type: every Krylov vector goes through the FP32 factors
// (z_k = M^-1 v_k with M = P^T L U, or L L^T), the product A z_k and the
// orthogonalisation run in the element type, and the correction is Z y.  A
// flexible method keeps the Arnoldi relation A Z = V H exact in the element
// type however coarse M is, so the residual it minimises is the true one.
// (Carson & Higham, "A new analysis of iterative refinement and its
// application to accurate solution of ill-conditioned sparse linear
// systems", SISC 2017; Haidar et al., SC18, for the tensor-core form.)
//
// Device work per inner step: the preconditioner (one gather and two
// single-launch triangular solves in FP32), one GEMV with A, classical
// Gram-Schmidt applied twice (CGS2) as two partial-dot and two update
// kernels -- deterministic fixed-partition reductions, no atomics -- and a
// scale kernel that also writes the next FP32 input.  The Hessenberg column
// and the norm come to the host (one small copy per step), where the Givens
// rotations and the least-squares update run in double.
#include "internal.cuh"

#include <cmath>
#include <vector>

namespace mgb {

constexpr int kKrylovThreads = 256;

static int parts_for(int64_t n) {
  int64_t p = (n + 4 * kKrylovThreads - 1) / (4 * kKrylovThreads);
  if (p < 1) p = 1;
  if (p > kKrylovMaxParts) p = kKrylovMaxParts;
  return (int)p;
}

template <typename S>
__device__ __forceinline__ double block_sum(double v, double *red) {
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int q = 0; q < kKrylovThreads / 32; q++) s += red[q];
  return s;  // valid in thread 0
}

// part[j * P + c] = sum over rows of part c of V(i, j) * w(i), j < k.
template <typename S>
__global__ void __launch_bounds__(kKrylovThreads)
    krylov_dots_kernel(int64_t n, int k, const S *__restrict__ V, int64_t ldv,
                       const S *__restrict__ w, double *__restrict__ part) {
  __shared__ double red[kKrylovThreads / 32];
  const int P = gridDim.x, c = blockIdx.x, j = blockIdx.y;
  const int64_t per = (n + P - 1) / P;
  const int64_t i0 = (int64_t)c * per;
  const int64_t i1 = i0 + per < n ? i0 + per : n;
  double s = 0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += kKrylovThreads)
    s += (double)V[i + j * ldv] * (double)w[i];
  s = block_sum<S>(s, red);
  if (threadIdx.x == 0) part[(int64_t)j * P + c] = s;
}

// h_j = sum_c part[j * P + c]; w -= V(:, 0:k) h; hout[j] (+)= h_j (block 0);
// when norm_part != null also part sums of the updated w^2 per block.
template <typename S>
__global__ void __launch_bounds__(kKrylovThreads)
    krylov_update_kernel(int64_t n, int k, const S *__restrict__ V, int64_t ldv,
                         const double *__restrict__ part, int P,
                         S *__restrict__ w, double *__restrict__ hout,
                         int accumulate, double *__restrict__ norm_part) {
  __shared__ double h[kKrylovMaxDim + 1];
  __shared__ double red[kKrylovThreads / 32];
  for (int j = threadIdx.x; j < k; j += kKrylovThreads) {
    double s = 0;
    for (int c = 0; c < P; c++) s += part[(int64_t)j * P + c];
    h[j] = s;
    if (blockIdx.x == 0) hout[j] = accumulate ? hout[j] + s : s;
  }
  __syncthreads();
  const int NB = gridDim.x;
  const int64_t per = (n + NB - 1) / NB;
  const int64_t i0 = (int64_t)blockIdx.x * per;
  const int64_t i1 = i0 + per < n ? i0 + per : n;
  double ss = 0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += kKrylovThreads) {
    double v = (double)w[i];
    for (int j = 0; j < k; j++) v -= (double)V[i + j * ldv] * h[j];
    w[i] = (S)v;
    ss += v * v;
  }
  if (norm_part) {
    ss = block_sum<S>(ss, red);
    if (threadIdx.x == 0) norm_part[blockIdx.x] = ss;
  }
}

// Part sums of w^2 (the initial residual's norm).
template <typename S>
__global__ void __launch_bounds__(kKrylovThreads)
    krylov_norm_kernel(int64_t n, const S *__restrict__ w,
                       double *__restrict__ norm_part) {
  __shared__ double red[kKrylovThreads / 32];
  const int NB = gridDim.x;
  const int64_t per = (n + NB - 1) / NB;
  const int64_t i0 = (int64_t)blockIdx.x * per;
  const int64_t i1 = i0 + per < n ? i0 + per : n;
  double ss = 0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += kKrylovThreads) {
    const double v = (double)w[i];
    ss += v * v;
  }
  ss = block_sum<S>(ss, red);
  if (threadIdx.x == 0) norm_part[blockIdx.x] = ss;
}

// Part maxima of |w| (NaN propagates).
template <typename S>
__global__ void __launch_bounds__(kKrylovThreads)
    krylov_amax_kernel(int64_t n, const S *__restrict__ w,
                       double *__restrict__ part) {
  __shared__ double red[kKrylovThreads / 32];
  const int NB = gridDim.x;
  const int64_t per = (n + NB - 1) / NB;
  const int64_t i0 = (int64_t)blockIdx.x * per;
  const int64_t i1 = i0 + per < n ? i0 + per : n;
  double m = 0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += kKrylovThreads) {
    const double v = fabs((double)w[i]);
    m = (v > m || v != v) ? v : m;
  }
  for (int off = 16; off; off >>= 1) {
    const double o = __shfl_xor_sync(0xffffffffu, m, off);
    m = (o > m || o != o) ? o : m;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0;
    for (int q = 0; q < kKrylovThreads / 32; q++) r = (red[q] > r || red[q] != red[q]) ? red[q] : r;
    part[blockIdx.x] = r;
  }
}

// v *= s (element type) and f = (float)v (the preconditioner's input).
template <typename S>
__global__ void krylov_scale_kernel(int64_t n, S *__restrict__ v, double s,
                                    float *__restrict__ f) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double t = (double)v[i] * s;
    v[i] = (S)t;
    f[i] = (float)t;
  }
}

template <typename S>
__global__ void krylov_widen_kernel(int64_t n, const float *__restrict__ f,
                                    S *__restrict__ z) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    z[i] = (S)f[i];
}

static unsigned grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  const int64_t cap = (int64_t)ctx()->sms * 8;
  return (unsigned)(g < 1 ? 1 : g > cap ? cap : g);
}

int fgmres_cycle(bool spd, int64_t n, const elem_t *A, int64_t lda,
                 const float *W, const int32_t *perm, elem_t *V, elem_t *Z,
                 float *F, int m, double rtol, double atol, int abort_after,
                 double abort_ratio, const KrylovTarget *tg, elem_t *d,
                 int *inner, double *res_est, int *stalled) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  cudaStream_t st = cx->stream;
  if (m > kKrylovMaxDim) m = kKrylovMaxDim;
  const int P = parts_for(n);
  const int NBU = P;  // blocks of the update / norm kernels
  // device scratch for partial sums and the Hessenberg column
  double *dpart = (double *)ws(WS_K, (size_t)(kKrylovMaxDim + 2) * kKrylovMaxParts *
                                         sizeof(double) * 2 + 4096);
  if (!dpart) return MATGB_ERR_NOMEM;
  double *dh = dpart + (size_t)(kKrylovMaxDim + 2) * kKrylovMaxParts;
  double *dnorm = dh + kKrylovMaxDim + 2;
  elem_t *y_dev = (elem_t *)(dnorm + kKrylovMaxParts);
  float *Fin = F, *Fout = F + n;
  std::vector<double> host(kKrylovMaxDim + 2 + kKrylovMaxParts);
  const unsigned g = grid_for(n);

  // beta = |r0|_2, v_1 = r0 / beta
  krylov_norm_kernel<elem_t><<<NBU, kKrylovThreads, 0, st>>>(n, V, dnorm);
  MGB_LAUNCHED("krylov_norm");
  MGB_CUDA(cudaMemcpyAsync(host.data(), dnorm, NBU * sizeof(double),
                           cudaMemcpyDeviceToHost, st));
  MGB_CUDA(cudaStreamSynchronize(st));
  double beta = 0;
  for (int c = 0; c < NBU; c++) beta += host[c];
  beta = std::sqrt(beta);
  *inner = 0;
  *res_est = beta;
  *stalled = 0;
  if (!(beta > 0) || !std::isfinite(beta)) {
    MGB_CUDA(cudaMemsetAsync(d, 0, (size_t)n * sizeof(elem_t), st));
    return 0;
  }
  krylov_scale_kernel<elem_t><<<g, 256, 0, st>>>(n, V, 1.0 / beta, Fin);
  MGB_LAUNCHED("krylov_scale");

  // Hessenberg (column-major, (m+1) x m), Givens rotations, rhs g
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), gv(m + 1, 0.0);
  gv[0] = beta;
  double target = std::fmax(rtol * beta, atol);
  std::vector<elem_t> ye(m);
  // d = Z y with y = R^-1 g over the first kc steps
  auto form_d = [&](int kc) -> int {
    std::vector<double> y(kc);
    for (int i = kc - 1; i >= 0; i--) {
      double t = gv[i];
      for (int j = i + 1; j < kc; j++) t -= H[(size_t)j * (m + 1) + i] * y[j];
      y[i] = t / H[(size_t)i * (m + 1) + i];
    }
    for (int i = 0; i < kc; i++) ye[i] = (elem_t)y[i];
    MGB_CUDA(cudaMemcpyAsync(y_dev, ye.data(), kc * sizeof(elem_t),
                             cudaMemcpyHostToDevice, st));
    MGB_TRY(gemv_t<elem_t>(n, kc, elem_t(1), Z, n, y_dev, elem_t(0), d));
    return 0;
  };
  int k = 0;
  for (; k < m; k++) {
    elem_t *zk = Z + (size_t)k * n;
    elem_t *w = V + (size_t)(k + 1) * n;
    // z_k = M^-1 v_k in FP32
    MGB_TRY(precond_solve(spd, n, W, perm, Fin, Fout));
    krylov_widen_kernel<elem_t><<<g, 256, 0, st>>>(n, Fout, zk);
    MGB_LAUNCHED("krylov_widen");
    // w = A z_k
    MGB_TRY(gemv_t<elem_t>(n, n, elem_t(1), A, lda, zk, elem_t(0), w));
    // CGS2 against v_0 .. v_k
    const int kk = k + 1;
    for (int pass = 0; pass < 2; pass++) {
      krylov_dots_kernel<elem_t><<<dim3(P, kk), kKrylovThreads, 0, st>>>(
          n, kk, V, n, w, dpart);
      MGB_LAUNCHED("krylov_dots");
      krylov_update_kernel<elem_t><<<NBU, kKrylovThreads, 0, st>>>(
          n, kk, V, n, dpart, P, w, dh, pass, pass == 1 ? dnorm : nullptr);
      MGB_LAUNCHED("krylov_update");
    }
    MGB_CUDA(cudaMemcpyAsync(host.data(), dh, kk * sizeof(double),
                             cudaMemcpyDeviceToHost, st));
    MGB_CUDA(cudaMemcpyAsync(host.data() + kKrylovMaxDim + 2, dnorm,
                             NBU * sizeof(double), cudaMemcpyDeviceToHost, st));
    MGB_CUDA(cudaStreamSynchronize(st));
    double hn = 0;
    for (int c = 0; c < NBU; c++) hn += host[kKrylovMaxDim + 2 + c];
    hn = std::sqrt(hn);
    double *col = &H[(size_t)k * (m + 1)];
    for (int j = 0; j < kk; j++) col[j] = host[j];
    col[kk] = hn;
    // previous rotations, then a new one zeroing col[k+1]
    for (int j = 0; j < k; j++) {
      const double t = cs[j] * col[j] + sn[j] * col[j + 1];
      col[j + 1] = -sn[j] * col[j] + cs[j] * col[j + 1];
      col[j] = t;
    }
    const double den = std::hypot(col[k], col[k + 1]);
    if (!(den > 0) || !std::isfinite(den)) break;  // breakdown or NaN
    cs[k] = col[k] / den;
    sn[k] = col[k + 1] / den;
    col[k] = den;
    col[k + 1] = 0;
    gv[k + 1] = -sn[k] * gv[k];
    gv[k] = cs[k] * gv[k];
    *res_est = std::fabs(gv[k + 1]);
    bool done = *res_est <= target || !(hn > 0);
    // every 8 steps of a first cycle: the correction so far gives |x|, and
    // with it the residual the backward-error target actually asks for
    if (!done && tg && (k + 1) % 8 == 0) {
      MGB_TRY(form_d(k + 1));
      krylov_amax_kernel<elem_t><<<NBU, kKrylovThreads, 0, st>>>(n, d, dnorm);
      MGB_LAUNCHED("krylov_amax");
      MGB_CUDA(cudaMemcpyAsync(host.data(), dnorm, NBU * sizeof(double),
                               cudaMemcpyDeviceToHost, st));
      MGB_CUDA(cudaStreamSynchronize(st));
      double xn = 0;
      for (int c = 0; c < NBU; c++) xn = (host[c] > xn || host[c] != host[c]) ? host[c] : xn;
      const double t2 = 0.25 * tg->tol * (tg->anorm * xn + tg->bnorm);
      if (t2 > target) target = t2;
      done = *res_est <= target;
    }
    // too slow for these factors: leave the cycle (the caller refactors)
    if (!done && k + 1 >= abort_after && *res_est > abort_ratio * beta) {
      *stalled = 1;
      k++;
      break;
    }
    if (!done && k + 1 < m) {
      krylov_scale_kernel<elem_t><<<g, 256, 0, st>>>(n, w, 1.0 / hn, Fin);
      MGB_LAUNCHED("krylov_scale");
    }
    if (done) {
      k++;
      break;
    }
  }
  *inner = k;
  // y = R^-1 g (k x k upper triangular), d = Z y
  if (k == 0) {
    MGB_CUDA(cudaMemsetAsync(d, 0, (size_t)n * sizeof(elem_t), st));
    return 0;
  }
  MGB_TRY(form_d(k));
  MGB_CUDA(cudaStreamSynchronize(st));  // ye is pageable host memory
  return 0;
}

}  // namespace mgb
