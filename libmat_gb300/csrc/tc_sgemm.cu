// FP32-accurate float GEMM and SYRK on the tensor cores.
//
// The plain float path of mat_mul / mat_gemm (mat.h:1842-1862, 2787-2796) and
// mat_syrk / mat_syrk_t (mat.h:5670-5679, 5727-5735): C = alpha*op(A)*op(B) +
// beta*C in mat.h's element type.  tcgen05 has no FP32 kind, so each operand
// is cut into two FP16 parts under a power-of-two scale per row of op(A) and
// per column of op(B):
//     s_i * op(A)_ik = Ah_ik + Al_ik,   t_j * op(B)_kj = Bh_jk + Bl_jk,
// with s_i chosen so that row i's largest magnitude lands in [2^14, 2^15)
// (FP16's top binade: the remainders stay normal down to 2^-3 and carry the
// next 11 bits).  The product of the split operands, without the Al*Bl term,
// is
//     Ah*Bh^T + Ah*Bl^T + Al*Bh^T  (three FP16 products, FP32 accumulation)
// and carries about 22 bits of each operand: FP32-level accuracy (the parity
// suite's product bound 2e-5 * K/256 of max |C|).  The three products run as
// one tcgen05 GEMM over a K axis of three segments (tc_gemm.cu), and the
// epilogue multiplies by 1/s_i and 1/t_j (exact) before alpha and beta.
//
// Packing: one pass finds the scale of every row of op(A) and column of op(B)
// (an order-preserving max of |x| as unsigned bits), a second converts and
// writes the FP16 parts K-contiguous, K padded with zeros to a multiple of 64
// (the TMA box); an operand stored with K as its slow index is transposed
// through shared memory on the way.
#include <cuda_fp16.h>

#include "internal.cuh"

namespace mgb {

namespace {

constexpr int kPackTile = 32;

// Largest |x| of row r of a rows x K operand into amax[r] (float bits, which
// order like the values for x >= 0; NaN rows compare largest).  contig: the
// operand element (r, kk) is at P[r*ld + kk] (else P[kk*ld + r]).
__global__ void pack_amax_kernel(int64_t rows, int64_t K,
                                 const float *__restrict__ P, int64_t ld,
                                 bool contig, unsigned *__restrict__ amax) {
  if (contig) {
    // one warp per row, lanes along K
    const int64_t r = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (r >= rows) return;
    const int lane = threadIdx.x & 31;
    unsigned m = 0;
    const float *row = P + r * ld;
    for (int64_t kk = lane; kk < K; kk += 32)
      m = max(m, __float_as_uint(fabsf(__ldg(row + kk))));
    for (int off = 16; off; off >>= 1) m = max(m, __shfl_xor_sync(~0u, m, off));
    if (lane == 0) amax[r] = m;
  } else {
    // threads along r (coalesced), blockIdx.y over chunks of K
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int64_t per = (K + gridDim.y - 1) / gridDim.y;
    const int64_t k0 = (int64_t)blockIdx.y * per;
    const int64_t k1 = k0 + per < K ? k0 + per : K;
    unsigned m = 0;
    for (int64_t kk = k0; kk < k1; kk++)
      m = max(m, __float_as_uint(fabsf(__ldg(P + kk * ld + r))));
    atomicMax(amax + r, m);
  }
}

// Power-of-two scale of a row whose largest magnitude has bits `a`: the scale
// that brings that magnitude into [2^14, 2^15); 1 for a zero or non-finite
// row (NaN and infinity then propagate as they would in FP32).
__device__ __forceinline__ int pack_exp(unsigned a) {
  const int e = (int)((a >> 23) & 0xFF);  // biased exponent of the max
  if (a == 0 || e == 0xFF) return 0;
  // max in [2^(e-127), 2^(e-126)); subnormal maxima count as 2^-126
  const int eb = e == 0 ? 1 : e;
  int sh = 14 - (eb - 127);
  if (sh > 127) sh = 127;
  if (sh < -126) sh = -126;
  return sh;
}

// v = hi + lo (two parts), or hi + mid + lo (three: mid null otherwise);
// each remainder is exact in FP32
__device__ __forceinline__ void split_store(float v, __half *hi, __half *mid,
                                            __half *lo, int64_t at) {
  const __half h = __float2half_rn(v);
  hi[at] = h;
  const float r = v - __half2float(h);
  if (mid) {
    const __half m = __float2half_rn(r);
    mid[at] = m;
    lo[at] = __float2half_rn(r - __half2float(m));
  } else {
    lo[at] = __float2half_rn(r);
  }
}

// Convert rows x K (scaled by 2^pack_exp(amax[r])) into hi / lo, row-major with
// leading dimension Kp (columns [K, Kp) zero); inv[r] = 2^-pack_exp.
// Contiguous operands: thread per element along K.  Transposed ones: a
// 32 x 32 tile through shared memory (read along r, write along K).
__global__ void pack_split_kernel(int64_t rows, int64_t K, int64_t Kp,
                                  const float *__restrict__ P, int64_t ld,
                                  bool contig, const unsigned *__restrict__ amax,
                                  __half *__restrict__ hi, __half *__restrict__ mid,
                                  __half *__restrict__ lo, float *__restrict__ inv) {
  __shared__ float tile[kPackTile][kPackTile + 1];
  const int64_t r0 = (int64_t)blockIdx.x * kPackTile;  // rows: grid x
  const int64_t k0 = (int64_t)blockIdx.y * kPackTile;  // K (<= 16384): grid y
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  if (!contig) {
    // tile[kk][r] = P[(k0+kk)*ld + r0 + r]
    for (int kk = ty; kk < kPackTile; kk += 8) {
      const int64_t gk = k0 + kk, gr = r0 + tx;
      tile[kk][tx] = (gk < K && gr < rows) ? __ldg(P + gk * ld + gr) : 0.f;
    }
    __syncthreads();
  }
  for (int rr = ty; rr < kPackTile; rr += 8) {
    const int64_t gr = r0 + rr, gk = k0 + tx;
    if (gr >= rows || gk >= Kp) continue;
    const int sh = pack_exp(__ldg(amax + gr));
    float v;
    if (contig)
      v = gk < K ? __ldg(P + gr * ld + gk) : 0.f;
    else
      v = tile[tx][rr];
    split_store(ldexpf(v, sh), hi, mid, lo, gr * Kp + gk);
    if (blockIdx.y == 0 && tx == 0) inv[gr] = ldexpf(1.f, -sh);
  }
}

struct Pack {
  __half *hi, *mid, *lo;  // mid null for two parts
  float *inv;
};

// Packs a rows x K operand into the FP16 split form: ws_slot holds the parts
// (parts * rows * Kp halves), inv and amax come from the caller's scratch.
int pack_operand(int64_t rows, int64_t K, int64_t Kp, const float *P, int64_t ld,
                 bool contig, int ws_slot, float *inv, unsigned *amax, int parts,
                 Pack *out) {
  cudaStream_t st = ctx()->stream;
  __half *h = (__half *)ws(ws_slot, (size_t)parts * rows * Kp * sizeof(__half));
  if (!h) return MATGB_ERR_NOMEM;
  __half *lo = h + rows * Kp;
  __half *md = parts == 3 ? h + 2 * rows * Kp : nullptr;
  MGB_CUDA(cudaMemsetAsync(amax, 0, (size_t)rows * sizeof(unsigned), st));
  {
    KtScope kt("tc_pack_amax", 0.0, 4.0 * rows * K);
    if (contig) {
      pack_amax_kernel<<<(unsigned)((rows + 7) / 8), 256, 0, st>>>(rows, K, P, ld,
                                                                  true, amax);
    } else {
      const int64_t rb = (rows + 255) / 256;
      int64_t kc = (int64_t)ctx()->sms * 8 / (rb > 0 ? rb : 1);
      if (kc < 1) kc = 1;
      if (kc > K) kc = K > 0 ? K : 1;
      if (kc > 65535) kc = 65535;
      pack_amax_kernel<<<dim3((unsigned)rb, (unsigned)kc), 256, 0, st>>>(
          rows, K, P, ld, false, amax);
    }
    MGB_LAUNCHED("tc_pack_amax");
  }
  {
    KtScope kt("tc_pack_split", 0.0, 4.0 * rows * K + 4.0 * rows * Kp);
    const dim3 g((unsigned)((rows + kPackTile - 1) / kPackTile),
                 (unsigned)((Kp + kPackTile - 1) / kPackTile));
    pack_split_kernel<<<g, 256, 0, st>>>(rows, K, Kp, P, ld, contig, amax, h, md,
                                         lo, inv);
    MGB_LAUNCHED("tc_pack_split");
  }
  out->hi = h;
  out->mid = md;
  out->lo = lo;
  out->inv = inv;
  return 0;
}

int g_plain_tc = 1;

}  // namespace

bool plain_tc_on() { return g_plain_tc != 0; }

// K is split into chunks of at most this many columns (each chunk one launch
// accumulating into C), which bounds a CTA's main loop (16384 columns in
// three segments, 8192 in six).
constexpr int64_t kSgemmKChunk = 16384;

int tc_sgemm(bool ta, bool tb, int64_t m, int64_t n, int64_t k, float alpha,
             const float *A, int64_t lda, const float *B, int64_t ldb,
             float beta, float *C, int64_t ldc, int tri, bool same_ab, int parts) {
  if (parts != 2 && parts != 3) return set_error(MATGB_ERR_ARG, "tc_sgemm: parts 2 or 3");
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (m <= 0 || n <= 0) return 0;
  if (m > INT32_MAX || n > INT32_MAX || m > (int64_t)65535 * 128 ||
      n > (int64_t)65535 * 256)
    return set_error(MATGB_ERR_ARG, "tc_sgemm: m or n too large");
  if (k <= 0 || alpha == 0.f) {
    // C = beta*C: the SIMT kernel handles the degenerate sums
    return gemm_skip_t<float>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C,
                              ldc, tri, nullptr);
  }
  const int64_t kchunk = parts == 3 ? kSgemmKChunk / 2 : kSgemmKChunk;
  for (int64_t kc0 = 0; kc0 < k; kc0 += kchunk) {
    const int64_t kc = k - kc0 < kchunk ? k - kc0 : kchunk;
    const int64_t Kp = (kc + 63) / 64 * 64;
    // the chunk's columns of op(A) (rows i, K-contiguous when ta) and rows of
    // op(B)^T (rows j: columns of op(B), K-contiguous when !tb)
    const float *Ac = ta ? A + kc0 : A + kc0 * lda;
    const float *Bc = tb ? B + kc0 * ldb : B + kc0;
    float *sc = (float *)ws(WS_TCS, (size_t)2 * (m + n) * sizeof(float));
    if (!sc) return MATGB_ERR_NOMEM;
    float *rinv = sc, *cinv = sc + m;
    unsigned *amax = reinterpret_cast<unsigned *>(sc + m + n);
    Pack pa, pb;
    MGB_TRY(pack_operand(m, kc, Kp, Ac, lda, ta, WS_TCA, rinv, amax, parts, &pa));
    if (same_ab) {
      pb = pa;
      pb.inv = rinv;
    } else {
      MGB_TRY(pack_operand(n, kc, Kp, Bc, ldb, !tb, WS_TCB, cinv, amax + m, parts,
                           &pb));
    }
    const float b = kc0 == 0 ? beta : 1.f;
    MGB_TRY(tc_gemm(0, m, n, Kp, pa.hi, Kp, pb.hi, Kp, alpha, nullptr, b, C, ldc,
                    tri, nullptr, pa.lo, pb.lo, rinv, same_ab ? rinv : cinv, pa.mid,
                    pb.mid));
  }
  return 0;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_plain_tensor_core(int on) {
  const int prev = g_plain_tc;
  if (on >= 0) g_plain_tc = on ? 1 : 0;
  return prev;
}

}  // extern "C"
