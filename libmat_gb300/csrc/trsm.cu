// Triangular solves with many right-hand sides (mat_solve_tril, _tril_unit,
// _triu, _trilt: mat.h:4580-4803; also the LU's U12 = L11^{-1} A12 step,
// mat.h:4264-4271).
//
// Blocked: diagonal blocks of up to kTrsmBlock rows are solved by one kernel
// with the block and 32 right-hand sides staged in shared memory (column-
// oriented substitution, the order of the reference's NEON tri-solves:
// x_j /= T_jj then x_i -= T_ij x_j); the off-diagonal updates are GEMMs.
#include "internal.cuh"

namespace mgb {

constexpr int kTrsmBlock = 96;
// 0: the blocked form below (diagonal-block kernel + GEMM updates) instead
// of the single-launch multi-RHS solver
static int g_trsm_flag = 1;
constexpr int kTrsmRhs = 32;

template <typename T>
static size_t trsm_smem(int tb) {
  return ((size_t)tb * (tb + 1) + (size_t)tb * (kTrsmRhs + 1)) * sizeof(T);
}

// Solves op(T)[0:tb,0:tb] X = B[0:tb, 32*blockIdx.x + 0..31] in place.
// EL: op(T) is lower triangular (forward), else upper (backward).
// TR: op(T) = T^T.  UNIT: unit diagonal (not read).
template <typename T, bool EL, bool TR, bool UNIT>
__global__ void __launch_bounds__(256)
    trsm_block_kernel(int tb, int64_t nrhs, const T *__restrict__ Tm,
                      int64_t ldt, T *__restrict__ B, int64_t ldb,
                      const int32_t *__restrict__ info) {
  if (info && *info != 0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *Rs = (T *)smem_raw;               // Rs[j*(tb+1)+i] = Tm[i + j*ldt]
  T *Xs = Rs + (size_t)tb * (tb + 1);  // Xs[i*33 + c]
  const int tid = threadIdx.x;
  const int c = tid & 31, g = tid >> 5;
  const int64_t c0 = (int64_t)blockIdx.x * kTrsmRhs;

  for (int e = tid; e < tb * tb; e += 256) {
    int i = e % tb, j = e / tb;
    Rs[j * (tb + 1) + i] = Tm[i + (int64_t)j * ldt];
  }
  for (int e = tid; e < tb * kTrsmRhs; e += 256) {
    int i = e % tb, cc = e / tb;
    int64_t col = c0 + cc;
    Xs[i * (kTrsmRhs + 1) + cc] = col < nrhs ? B[i + col * ldb] : T(0);
  }
  __syncthreads();
  auto Te = [&](int i, int j) -> T {
    return TR ? Rs[i * (tb + 1) + j] : Rs[j * (tb + 1) + i];
  };
  constexpr int LD = kTrsmRhs + 1;
  if (EL) {
    if (!UNIT && g == 0) Xs[c] = Xs[c] / Te(0, 0);
    __syncthreads();
    for (int k = 0; k < tb; k++) {
      const T xk = Xs[k * LD + c];
      for (int i = k + 1 + g; i < tb; i += 8) {
        T v = fma(-Te(i, k), xk, Xs[i * LD + c]);
        if (!UNIT && i == k + 1) v = v / Te(i, i);
        Xs[i * LD + c] = v;
      }
      __syncthreads();
    }
  } else {
    if (!UNIT && g == 0)
      Xs[(tb - 1) * LD + c] = Xs[(tb - 1) * LD + c] / Te(tb - 1, tb - 1);
    __syncthreads();
    for (int k = tb - 1; k >= 0; k--) {
      const T xk = Xs[k * LD + c];
      for (int i = k - 1 - g; i >= 0; i -= 8) {
        T v = fma(-Te(i, k), xk, Xs[i * LD + c]);
        if (!UNIT && i == k - 1) v = v / Te(i, i);
        Xs[i * LD + c] = v;
      }
      __syncthreads();
    }
  }
  for (int e = tid; e < tb * kTrsmRhs; e += 256) {
    int i = e % tb, cc = e / tb;
    int64_t col = c0 + cc;
    if (col < nrhs) B[i + col * ldb] = Xs[i * LD + cc];
  }
}

template <typename T, bool EL, bool TR, bool UNIT>
static int launch_block(int tb, int64_t nrhs, const T *Tm, int64_t ldt, T *B,
                        int64_t ldb, const int32_t *info) {
  static bool attr_set = false;
  auto k = trsm_block_kernel<T, EL, TR, UNIT>;
  if (!attr_set) {
    MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)trsm_smem<T>(kTrsmBlock)));
    attr_set = true;
  }
  unsigned grid = (unsigned)((nrhs + kTrsmRhs - 1) / kTrsmRhs);
  KtScope kt("trsm_block", (double)tb * tb * nrhs,
             (double)sizeof(T) * (tb * tb / 2.0 + 2.0 * tb * nrhs));
  k<<<grid, 256, trsm_smem<T>(tb), ctx()->stream>>>(tb, nrhs, Tm, ldt, B, ldb,
                                                     info);
  MGB_LAUNCHED("trsm_block");
  return 0;
}

template <typename T>
static int block_solve(bool el, bool tr, bool unit, int tb, int64_t nrhs,
                       const T *Tm, int64_t ldt, T *B, int64_t ldb,
                       const int32_t *info) {
#define MGB_B(E, R, U)                                                         \
  if (el == E && tr == R && unit == U)                                         \
    return launch_block<T, E, R, U>(tb, nrhs, Tm, ldt, B, ldb, info);
  MGB_B(true, false, false)
  MGB_B(true, false, true)
  MGB_B(true, true, false)
  MGB_B(true, true, true)
  MGB_B(false, false, false)
  MGB_B(false, false, true)
  MGB_B(false, true, false)
  MGB_B(false, true, true)
#undef MGB_B
  return MATGB_ERR_ARG;
}

template <typename T>
int trsm_left_t(bool lower, bool trans, bool unit, int64_t n, int64_t nrhs,
                const T *Tm, int64_t ldt, T *B, int64_t ldb,
                const int32_t *info) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  if (n <= 0 || nrhs <= 0) return 0;
  // one right-hand side: the single-launch solver (no failure flag to honour);
  // several: the single-launch multi-RHS solver
  if (nrhs == 1 && !info) return trsv_t<T>(lower, trans, unit, n, Tm, ldt, B);
  if (g_trsm_flag) return trsm_flag_t<T>(lower, trans, unit, n, nrhs, Tm, ldt, B, ldb, info);
  const bool el = (lower != trans);
  // Pointer to op(T)(r0, c0) for use as a GEMM operand with transpose 'trans'.
  auto sub = [&](int64_t r0, int64_t c0) {
    return trans ? Tm + c0 + r0 * ldt : Tm + r0 + c0 * ldt;
  };
  if (el) {
    for (int64_t ib = 0; ib < n; ib += kTrsmBlock) {
      int tb = (int)((n - ib) < kTrsmBlock ? (n - ib) : kTrsmBlock);
      MGB_TRY(block_solve<T>(el, trans, unit, tb, nrhs, Tm + ib + ib * ldt,
                             ldt, B + ib, ldb, info));
      if (ib + tb < n)
        MGB_TRY(gemm_skip_t<T>(trans, false, n - ib - tb, nrhs, tb, T(-1),
                               sub(ib + tb, ib), ldt, B + ib, ldb, T(1),
                               B + ib + tb, ldb, 0, info));
    }
  } else {
    int64_t last = ((n - 1) / kTrsmBlock) * kTrsmBlock;
    for (int64_t ib = last; ib >= 0; ib -= kTrsmBlock) {
      int tb = (int)((n - ib) < kTrsmBlock ? (n - ib) : kTrsmBlock);
      MGB_TRY(block_solve<T>(el, trans, unit, tb, nrhs, Tm + ib + ib * ldt,
                             ldt, B + ib, ldb, info));
      if (ib > 0)
        MGB_TRY(gemm_skip_t<T>(trans, false, ib, nrhs, tb, T(-1), sub(0, ib),
                               ldt, B + ib, ldb, T(1), B, ldb, 0, info));
    }
  }
  return 0;
}

template int trsm_left_t<float>(bool, bool, bool, int64_t, int64_t,
                                const float *, int64_t, float *, int64_t,
                                const int32_t *);
template int trsm_left_t<double>(bool, bool, bool, int64_t, int64_t,
                                 const double *, int64_t, double *, int64_t,
                                 const int32_t *);

int trsm_left(bool lower, bool trans, bool unit, int64_t n, int64_t nrhs,
              const elem_t *T, int64_t ldt, elem_t *B, int64_t ldb,
              const int32_t *info) {
  return trsm_left_t<elem_t>(lower, trans, unit, n, nrhs, T, ldt, B, ldb, info);
}

}  // namespace mgb

using namespace mgb;

extern "C" int matgb_trsm_dev(char uplo, char trans, char diag, size_t n,
                              size_t nrhs, const mat_elem_t *T, size_t ldt,
                              mat_elem_t *B, size_t ldb) {
  bool lower = (uplo == 'L' || uplo == 'l');
  bool upper = (uplo == 'U' || uplo == 'u');
  bool tr = (trans == 'T' || trans == 't');
  bool unit = (diag == 'U' || diag == 'u');
  if ((!lower && !upper) || (!tr && trans != 'N' && trans != 'n') ||
      (!unit && diag != 'N' && diag != 'n'))
    return set_error(MATGB_ERR_ARG, "trsm: bad uplo/trans/diag");
  if (ldt < n || ldb < n)
    return set_error(MATGB_ERR_ARG, "trsm: leading dimension too small");
  return trsm_left(lower, tr, unit, (int64_t)n, (int64_t)nrhs, T, (int64_t)ldt,
                   B, (int64_t)ldb, nullptr);
}
