// Tensor-core rank-K update for the mixed-precision factorisations:
//     C (fp32, column-major) = beta*C + alpha * A * B^T
// with A (M x K) and B (N x K) in BF16 or FP16, both K-contiguous.
//
// This is the low-precision form of the LU trailing update A22 -= L21*U12
// (mat__gemm_strided_ call at mat.h:4277-4283) and of the Cholesky SYRK
// update (mat.h:6021-6023): the bulk of the FLOPs run on the 5th-generation
// tensor cores with FP32 accumulation in TMEM, the trailing matrix stays FP32.
//
// Split form (three products): with A = Ah + Al and B = Bh + Bl (16-bit hi
// parts and the rounding remainders), A B^T ~= Ah Bh^T + Ah Bl^T + Al Bh^T,
// the dropped Al Bl^T being ~2^-22 of the product -- FP32-level updates from
// FP16 tensor cores.  The three products are one GEMM over a K axis of three
// segments, [Ah|Ah|Al] . [Bh|Bl|Bh]^T: the producer picks the hi or lo tensor
// map per segment, so C is read and written once.
//
// One CTA computes one 128 x 256 tile (UMMA M=128, N=256, K=16, cta_group::1):
//   warp 8  : TMA producer -- for each 64-wide K block a 128x64 A box and a
//             256x64 B box (128-byte swizzle) into a ring of 2 stages (short
//             K, two CTAs per SM) or 4 (long K, one CTA per SM) with full /
//             empty mbarriers;
//   warp 9  : TMEM allocator and single-thread MMA issuer (4 MMAs per K
//             block, tcgen05.commit to the stage's empty barrier), then a
//             final commit to the "accumulator ready" mbarrier;
//   warps 0-7: epilogue -- tcgen05.ld 16 columns at a time from TMEM (warp w
//             reads lane quarter w%4, column half w/4), then a coalesced
//             read-modify-write of C (consecutive lanes = consecutive rows).
// The 2-stage form takes 96 KB of smem, so two CTAs fit per SM and one CTA's
// epilogue overlaps the other's loads and MMAs; the 4-stage form (192 KB)
// serves long K sums, where the epilogue is a few percent of a tile.  Every wait is bounded; on a timeout the CTA records
// an error flag, stops issuing work, waits (bounded) for its copies in
// flight, still frees its TMEM and returns.
#include <cudaTypedefs.h>

#include <initializer_list>

#include "internal.cuh"
#include "tc_ptx.cuh"

namespace mgb {

constexpr int kTcBM = 128, kTcBN = 256, kTcBK = 64;
constexpr int kTcThreads = 320;
constexpr uint32_t kTcWaitLimit = 1u << 24;  // ~1.5 s of polling
// producer / MMA polls before sleeping, and whether the epilogue pulls its C
// region towards L2 during the main loop (build-time overrides for
// measurement: -DMGB_TC_SPIN=n, -DMGB_TC_PREFETCH=1).  Measured on the split
// update at 16000 x 15856 x 192: 0.574 ms spinning, 0.579 ms sleeping from
// the first poll; the L2 prefetch took it to 0.588 ms (the chunked loads
// already overlap the other CTA's main loop), so it is off.
#ifndef MGB_TC_SPIN
#define MGB_TC_SPIN 256
#endif
#ifndef MGB_TC_PREFETCH
#define MGB_TC_PREFETCH 0
#endif
constexpr uint32_t kTcSpin = MGB_TC_SPIN;
// K blocks per launch (all segments): bounds one CTA's main loop (3 x 16384
// columns of K, ~0.3 ms on one SM), far inside the wait limit; longer sums
// are split by the caller
constexpr int kTcMaxKB = 3 * 16384 / kTcBK;

// Two ring depths: 2 stages with two CTAs per SM (short K, up to 32 K blocks
// over all segments: the LU and Cholesky updates, where one CTA's epilogue
// overlaps the other's main loop), and 4 stages with one CTA per SM (long K,
// the plain GEMM: deeper prefetch).
template <int ST>
struct TcSmem {
  // 1024-byte aligned swizzle atoms
  uint16_t a[ST][kTcBM * kTcBK];
  uint16_t b[ST][kTcBN * kTcBK];
  uint64_t full[ST];
  uint64_t empty[ST];
  uint64_t done;
  uint32_t tmem_base;
  volatile int timeout;
};

// Segment s of the K axis (kps K blocks each) reads A from map (amask >> 2s)
// & 3 of tmA0 / tmA1 / tmA2, B likewise from bmask (up to 6 segments).
// tri: 0 every tile; 1 lower (tiles on/below the diagonal, elements with
// col <= row); 2 upper (col >= row).  rinv / cinv (may be null): per-row and
// per-column power-of-two factors applied to the accumulator before alpha
// (the inverses of the operands' packing scales; exact).
template <int ST, int MINB, bool SC>
__global__ void __launch_bounds__(kTcThreads, MINB)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA0,
                   const __grid_constant__ CUtensorMap tmA1,
                   const __grid_constant__ CUtensorMap tmA2,
                   const __grid_constant__ CUtensorMap tmB0,
                   const __grid_constant__ CUtensorMap tmB1,
                   const __grid_constant__ CUtensorMap tmB2, int M, int N,
                   int kps, int nseg, unsigned amask, unsigned bmask,
                   float alpha, const float *__restrict__ alpha_scale,
                   float beta, float *__restrict__ C, int64_t ldc,
                   uint32_t idesc, int tri, const int32_t *__restrict__ skip,
                   const float *__restrict__ rinv,
                   const float *__restrict__ cinv, int *__restrict__ err) {
  constexpr int kTcStages = ST;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // align the carve-out to 1024 B (the swizzle atom)
  TcSmem<ST> &s = *reinterpret_cast<TcSmem<ST> *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kTcBM, n0 = blockIdx.y * kTcBN;
  const int nkb = kps * nseg;
  // whole-CTA exits before any barrier or TMEM allocation: a failed earlier
  // step (skip flag) or a tile strictly outside the triangle
  if (skip && *skip != 0) return;
  if (tri == 1 && n0 >= m0 + kTcBM) return;
  if (tri == 2 && m0 >= n0 + kTcBN) return;

  if (threadIdx.x == 0) {
    for (int i = 0; i < kTcStages; i++) {
      tc::mbar_init(&s.full[i], 1);
      tc::mbar_init(&s.empty[i], 1);
    }
    tc::mbar_init(&s.done, 1);
    s.timeout = 0;
    tc::fence_barrier_init();
  }
  if (warp == 9) tc::tmem_alloc(&s.tmem_base, kTcBN);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = s.tmem_base;

  if (warp == 8 && lane == 0) {
    tc::prefetch_tmap(&tmA0);
    tc::prefetch_tmap(&tmB0);
    int issued = 0;
    for (int kb = 0; kb < nkb; kb++) {
      const int st = kb % kTcStages, use = kb / kTcStages;
      if (use > 0 && !tc::mbar_wait(&s.empty[st], (use - 1) & 1, kTcWaitLimit, kTcSpin)) {
        s.timeout = 1;
        break;
      }
      if (s.timeout) break;
      const int seg = kb / kps, kx = (kb % kps) * kTcBK;
      const unsigned sa = (amask >> (2 * seg)) & 3u, sb = (bmask >> (2 * seg)) & 3u;
      const CUtensorMap *ma = sa == 2 ? &tmA2 : sa == 1 ? &tmA1 : &tmA0;
      const CUtensorMap *mb = sb == 2 ? &tmB2 : sb == 1 ? &tmB1 : &tmB0;
      tc::mbar_arrive_expect_tx(&s.full[st], (kTcBM + kTcBN) * kTcBK * 2);
      tc::tma_load_2d(s.a[st], ma, kx, m0, &s.full[st]);
      tc::tma_load_2d(s.b[st], mb, kx, n0, &s.full[st]);
      issued = kb + 1;
    }
    // no copy may still be in flight when the CTA leaves: wait (bounded) for
    // the last load issued into each stage
    for (int kb = issued - kTcStages > 0 ? issued - kTcStages : 0; kb < issued; kb++)
      tc::mbar_wait(&s.full[kb % kTcStages], (kb / kTcStages) & 1, kTcWaitLimit);
  } else if (warp == 9 && lane == 0) {
    bool ok = true;
    for (int kb = 0; kb < nkb; kb++) {
      const int st = kb % kTcStages, use = kb / kTcStages;
      if (s.timeout || !tc::mbar_wait(&s.full[st], use & 1, kTcWaitLimit, kTcSpin)) {
        ok = false;
        break;
      }
      tc::tc_fence_after();
      const uint32_t a0 = tc::smem_u32(s.a[st]), b0 = tc::smem_u32(s.b[st]);
#pragma unroll
      for (int kk = 0; kk < kTcBK / 16; kk++) {
        // advance 16 elements (32 bytes) along K inside the 128-byte atom
        const uint64_t ad = tc::desc_k_sw128(a0 + kk * 32);
        const uint64_t bd = tc::desc_k_sw128(b0 + kk * 32);
        tc::mma_f16(tmem, ad, bd, idesc, (kb | kk) ? 1u : 0u);
      }
      tc::mma_commit(&s.empty[st]);  // the stage is free once these finish
    }
    if (ok) {
      tc::mma_commit(&s.done);
    } else {
      // the commit still fires once the MMAs already issued have finished,
      // so TMEM is not freed under them
      s.timeout = 1;
      atomicExch(err, 1);
      tc::mma_commit(&s.done);
    }
  } else if (warp < 8) {
    // Epilogue: warp w reads TMEM lane quarter w%4 (rows q*32..q*32+31) and
    // column half w/4, in 16-column chunks; the C values of the next chunk are
    // loaded before the current one is finished (the first before the
    // accumulator is even ready), so HBM latency overlaps the MMAs.
    constexpr int CH = 16, NCH = kTcBN / 2 / CH;
    const int q = warp & 3, half = warp >> 2;
    const int row = m0 + q * 32 + lane;
    const int cbase = n0 + half * (kTcBN / 2);
    const bool rok = row < M;
    const bool rd = beta != 0.f;
    float *cp = C + (int64_t)cbase * ldc + row;
    auto load = [&](float (&d)[CH], int ch) {
#pragma unroll
      for (int j = 0; j < CH; j++) {
        const int col = ch * CH + j;
        d[j] = (rok && rd && cbase + col < N) ? cp[(int64_t)col * ldc] : 0.f;
      }
    };
    // Pull this warp's whole C region (32 rows x 128 columns, one 128-byte
    // line per column) towards L2 while the MMAs run, so the chunk loads
    // below find it there: the DRAM reads of C overlap the main loop
    // instead of the epilogue.
    if (MGB_TC_PREFETCH && rd) {
      const int row0 = m0 + q * 32;
      if (row0 < M) {
        const float *c0 = C + (int64_t)cbase * ldc + row0;
#pragma unroll
        for (int j = lane; j < kTcBN / 2; j += 32)
          if (cbase + j < N && (tri != 1 || cbase + j <= row0 + 31) &&
              (tri != 2 || cbase + j >= row0))
            tc::prefetch_l2(c0 + (int64_t)j * ldc);
      }
    }
    float cur[CH];
    load(cur, 0);
    float rs = 1.f;
    if constexpr (SC) rs = (rok && rinv) ? __ldg(&rinv[row]) : 1.f;
    const bool ready = tc::mbar_wait(&s.done, 0, kTcWaitLimit);
    tc::tc_fence_after();
    if (ready && !s.timeout) {
      const float al = alpha_scale ? alpha * (*alpha_scale) : alpha;
#pragma unroll 1
      for (int ch = 0; ch < NCH; ch++) {
        float nxt[CH];
        if (ch + 1 < NCH) load(nxt, ch + 1);
        float cs[CH];
        if constexpr (SC) {
#pragma unroll
          for (int j = 0; j < CH; j++) {
            const int col = cbase + ch * CH + j;
            cs[j] = col < N ? __ldg(&cinv[col]) : 1.f;
          }
        }
        float v[CH];
        tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) +
                          (uint32_t)(half * (kTcBN / 2) + ch * CH),
                      v);
        if (rok) {
#pragma unroll
          for (int j = 0; j < CH; j++) {
            const int col = ch * CH + j;
            const bool in = tri == 0 || (tri == 1 ? cbase + col <= row
                                                   : cbase + col >= row);
            if (cbase + col < N && in) {
              if constexpr (SC)
                cp[(int64_t)col * ldc] = fmaf(al, (v[j] * rs) * cs[j], beta * cur[j]);
              else
                cp[(int64_t)col * ldc] = fmaf(al, v[j], beta * cur[j]);
            }
          }
        }
        if (ch + 1 < NCH) {
#pragma unroll
          for (int j = 0; j < CH; j++) cur[j] = nxt[j];
        }
      }
    } else if (!ready) {
      atomicExch(err, 2);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 9) {
    __syncwarp();
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, kTcBN);
  }
}

// ---- persistent form (short K: the trailing updates) ------------------------
// One CTA per SM pulls 128 x 256 tiles from a per-stream counter (dynamic, so
// CTAs that start late -- behind the LU's panel kernel on some SMs -- take
// fewer tiles), through a 4-stage ring, with two TMEM accumulators: the
// epilogue of tile i (8 warps, three C chunks in flight per thread) runs
// under the main loop of tile i+1.  Warp 8 lane 0 takes the tile indices and
// issues the TMA loads; warp 9 allocates TMEM (512 columns) and issues the
// MMAs; the tile indices reach the MMA thread and the epilogue warps through
// a 4-slot ring.  Every wait is bounded as in tc_gemm_kernel.
constexpr int kTcPTiles = 4;

template <int BN, int ST>
struct TcPSmem {
  uint16_t a[ST][kTcBM * kTcBK];
  uint16_t b[ST][BN * kTcBK];
  uint64_t full[ST];
  uint64_t empty[ST];
  uint64_t acc_full[2];
  uint64_t acc_empty[2];
  uint64_t tfull[kTcPTiles];
  uint64_t tempty[kTcPTiles];
  uint64_t drain;
  int tile[kTcPTiles];
  uint32_t tmem_base;
  volatile int timeout;
};

template <bool SC, int BN, int ST, int MINB>
__global__ void __launch_bounds__(kTcThreads, MINB)
    tc_gemm_pkernel(const __grid_constant__ CUtensorMap tmA0,
                    const __grid_constant__ CUtensorMap tmA1,
                    const __grid_constant__ CUtensorMap tmA2,
                    const __grid_constant__ CUtensorMap tmB0,
                    const __grid_constant__ CUtensorMap tmB1,
                    const __grid_constant__ CUtensorMap tmB2, int M, int N,
                    int kps, int nseg, unsigned amask, unsigned bmask,
                    float alpha, const float *__restrict__ alpha_scale,
                    float beta, float *__restrict__ C, int64_t ldc,
                    uint32_t idesc, int tri, const int32_t *__restrict__ skip,
                    const float *__restrict__ rinv, const float *__restrict__ cinv,
                    int *__restrict__ err, int mtiles, int ntiles,
                    int *__restrict__ ctr) {
  extern __shared__ __align__(1024) unsigned char tcp_smem[];
  constexpr int kTcPStages = ST;
  TcPSmem<BN, ST> &s = *reinterpret_cast<TcPSmem<BN, ST> *>(
      tcp_smem + ((1024u - (tc::smem_u32(tcp_smem) & 1023u)) & 1023u));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkb = kps * nseg, ntot = mtiles * ntiles;
  if (skip && *skip != 0) return;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kTcPStages; i++) {
      tc::mbar_init(&s.full[i], 1);
      tc::mbar_init(&s.empty[i], 1);
    }
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(&s.acc_full[i], 1);
      tc::mbar_init(&s.acc_empty[i], 8);
    }
    for (int i = 0; i < kTcPTiles; i++) {
      tc::mbar_init(&s.tfull[i], 1);
      tc::mbar_init(&s.tempty[i], 9);
    }
    tc::mbar_init(&s.drain, 1);
    s.timeout = 0;
    tc::fence_barrier_init();
  }
  if (warp == 9) tc::tmem_alloc(&s.tmem_base, 2 * BN);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = s.tmem_base;

  if (warp == 8 && lane == 0) {
    // ---- tile indices and TMA loads
    tc::prefetch_tmap(&tmA0);
    tc::prefetch_tmap(&tmB0);
    int g = 0;
    for (int i = 0;; i++) {
      const int slot = i % kTcPTiles, use = i / kTcPTiles;
      if (use > 0 && !tc::mbar_wait(&s.tempty[slot], (use - 1) & 1, kTcWaitLimit, kTcSpin)) {
        s.timeout = 1;
        break;
      }
      int t = -1;
      while (!s.timeout) {
        const int c = atomicAdd(ctr, 1);
        if (c >= ntot) break;
        const int m0 = (c % mtiles) * kTcBM, n0 = (c / mtiles) * BN;
        if (tri == 1 && n0 >= m0 + kTcBM) continue;  // strictly above the diagonal
        if (tri == 2 && m0 >= n0 + BN) continue;
        t = c;
        break;
      }
      s.tile[slot] = t;
      tc::mbar_arrive(&s.tfull[slot]);
      if (t < 0) break;
      const int m0 = (t % mtiles) * kTcBM, n0 = (t / mtiles) * BN;
      for (int kb = 0; kb < nkb; kb++, g++) {
        const int st = g % kTcPStages, u = g / kTcPStages;
        if (u > 0 && !tc::mbar_wait(&s.empty[st], (u - 1) & 1, kTcWaitLimit, kTcSpin)) {
          s.timeout = 1;
          break;
        }
        if (s.timeout) break;
        const int seg = kb / kps, kx = (kb % kps) * kTcBK;
        const unsigned sa = (amask >> (2 * seg)) & 3u, sb = (bmask >> (2 * seg)) & 3u;
        const CUtensorMap *ma = sa == 2 ? &tmA2 : sa == 1 ? &tmA1 : &tmA0;
        const CUtensorMap *mb = sb == 2 ? &tmB2 : sb == 1 ? &tmB1 : &tmB0;
        tc::mbar_arrive_expect_tx(&s.full[st], (kTcBM + BN) * kTcBK * 2);
        tc::tma_load_2d(s.a[st], ma, kx, m0, &s.full[st]);
        tc::tma_load_2d(s.b[st], mb, kx, n0, &s.full[st]);
      }
      if (s.timeout) break;
    }
    // no copy may still be in flight when the CTA leaves
    for (int q = g - kTcPStages > 0 ? g - kTcPStages : 0; q < g; q++)
      tc::mbar_wait(&s.full[q % kTcPStages], (q / kTcPStages) & 1, kTcWaitLimit);
  } else if (warp == 9 && lane == 0) {
    // ---- MMAs into accumulator i % 2
    int g = 0;
    bool issued = false;
    for (int i = 0;; i++) {
      const int slot = i % kTcPTiles, use = i / kTcPTiles;
      if (!tc::mbar_wait(&s.tfull[slot], use & 1, kTcWaitLimit, kTcSpin)) {
        s.timeout = 1;
        atomicExch(err, 1);
        break;
      }
      const int t = s.tile[slot];
      tc::mbar_arrive(&s.tempty[slot]);
      if (t < 0 || s.timeout) break;
      const int a = i & 1, au = i >> 1;
      if (au > 0 && !tc::mbar_wait(&s.acc_empty[a], (au - 1) & 1, kTcWaitLimit, kTcSpin)) {
        s.timeout = 1;
        atomicExch(err, 1);
        break;
      }
      tc::tc_fence_after();
      const uint32_t acc = tmem + (uint32_t)(a * BN);
      bool ok = true;
      for (int kb = 0; kb < nkb; kb++, g++) {
        const int st = g % kTcPStages, u = g / kTcPStages;
        if (s.timeout || !tc::mbar_wait(&s.full[st], u & 1, kTcWaitLimit, kTcSpin)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t a0 = tc::smem_u32(s.a[st]), b0 = tc::smem_u32(s.b[st]);
#pragma unroll
        for (int kk = 0; kk < kTcBK / 16; kk++)
          tc::mma_f16(acc, tc::desc_k_sw128(a0 + kk * 32), tc::desc_k_sw128(b0 + kk * 32),
                      idesc, (kb | kk) ? 1u : 0u);
        issued = true;
        tc::mma_commit(&s.empty[st]);
      }
      tc::mma_commit(&s.acc_full[a]);
      if (!ok) {
        s.timeout = 1;
        atomicExch(err, 1);
        break;
      }
    }
    // every MMA this thread issued has finished before TMEM is freed
    if (issued) {
      tc::mma_commit(&s.drain);
      tc::mbar_wait(&s.drain, 0, kTcWaitLimit);
    }
  } else if (warp < 8) {
    // ---- epilogue: warp w reads TMEM lane quarter w%4, column half w/4
    constexpr int CH = 16, NCH = BN / 2 / CH;
    const int q = warp & 3, half = warp >> 2;
    const bool rd = beta != 0.f;
    for (int i = 0;; i++) {
      const int slot = i % kTcPTiles, use = i / kTcPTiles;
      if (!tc::mbar_wait(&s.tfull[slot], use & 1, kTcWaitLimit)) {
        atomicExch(err, 2);
        break;
      }
      const int t = s.tile[slot];
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&s.tempty[slot]);
      if (t < 0 || s.timeout) break;
      const int m0 = (t % mtiles) * kTcBM, n0 = (t / mtiles) * BN;
      const int row = m0 + q * 32 + lane;
      const int cbase = n0 + half * (BN / 2);
      const bool rok = row < M;
      float *cp = C + (int64_t)cbase * ldc + row;
      auto load = [&](float (&d)[CH], int ch) {
#pragma unroll
        for (int j = 0; j < CH; j++) {
          const int col = ch * CH + j;
          d[j] = (rok && rd && cbase + col < N) ? cp[(int64_t)col * ldc] : 0.f;
        }
      };
      // C chunks 0 and 1 in flight before the accumulator is ready, and two
      // ahead of the one being finished after that
      float c0[CH], c1[CH];
      load(c0, 0);
      if (NCH > 1) load(c1, 1);
      float rs = 1.f;
      if constexpr (SC) rs = (rok && rinv) ? __ldg(&rinv[row]) : 1.f;
      const int a = i & 1, au = i >> 1;
      const bool ready = tc::mbar_wait(&s.acc_full[a], au & 1, kTcWaitLimit);
      tc::tc_fence_after();
      if (!ready) {
        atomicExch(err, 2);
        break;
      }
      const float al = alpha_scale ? alpha * (*alpha_scale) : alpha;
#pragma unroll 1
      for (int ch = 0; ch < NCH; ch++) {
        float c2[CH];
        if (ch + 2 < NCH) load(c2, ch + 2);
        float v[CH];
        tc::tmem_ld16(tmem + (uint32_t)(a * BN) + ((uint32_t)(q * 32) << 16) +
                          (uint32_t)(half * (BN / 2) + ch * CH),
                      v);
        if (rok) {
#pragma unroll
          for (int j = 0; j < CH; j++) {
            const int col = ch * CH + j;
            const bool in = tri == 0 || (tri == 1 ? cbase + col <= row : cbase + col >= row);
            if (cbase + col < N && in) {
              // (the column's scale read here, not staged: the two-CTA
              // register budget)
              if constexpr (SC)
                cp[(int64_t)col * ldc] =
                    fmaf(al, (v[j] * rs) * __ldg(&cinv[cbase + col]), beta * c0[j]);
              else
                cp[(int64_t)col * ldc] = fmaf(al, v[j], beta * c0[j]);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < CH; j++) {
          c0[j] = c1[j];
          c1[j] = c2[j];
        }
      }
      // this accumulator is read: the MMAs of tile i+2 may overwrite it
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&s.acc_empty[a]);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 9) {
    __syncwarp();
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 2 * BN);
  }
}

// ---- host side ----------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static int *g_tc_err = nullptr;
static bool g_tc_ready = false;
// The persistent form's tile counters, one per stream that launches it (the
// launches of one stream are ordered, so each is zeroed before its launch
// without racing another launch that still uses it).
constexpr int kTcCtrs = 32;
static int *g_tc_ctr = nullptr;
static cudaStream_t g_tc_ctr_stream[kTcCtrs];
static int g_tc_nctr = 0;
static int *tile_counter(cudaStream_t st) {
  for (int i = 0; i < g_tc_nctr; i++)
    if (g_tc_ctr_stream[i] == st) return g_tc_ctr + i;
  if (g_tc_nctr == kTcCtrs) return nullptr;
  g_tc_ctr_stream[g_tc_nctr] = st;
  return g_tc_ctr + g_tc_nctr++;
}
// 1 (default): short-K products take the persistent form; 0: the 2-stage
// two-CTAs-per-SM form (matgb_tc_persistent).
static int g_tc_persistent = 1;
// the persistent form's tile width and ring depth: two CTAs per SM
// (2 x 3 stages x 32 KB of shared memory, 2 x 2 x 128 TMEM columns)
constexpr int kTcPBN = 128, kTcPST = 3;

template <int ST>
static constexpr size_t tc_smem_bytes() {
  return sizeof(TcSmem<ST>) + 1024;
}

static int tc_setup() {
  if (g_tc_ready) return 0;
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  MGB_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn,
                                            12000, cudaEnableDefault, &q));
  if (!fn || q != cudaDriverEntryPointSuccess)
    return set_error(MATGB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  MGB_CUDA(cudaMalloc(&g_tc_err, sizeof(int)));
  MGB_CUDA(cudaMemset(g_tc_err, 0, sizeof(int)));
  MGB_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<2, 2, false>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tc_smem_bytes<2>()));
  MGB_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<2, 2, true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tc_smem_bytes<2>()));
  MGB_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<4, 1, false>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tc_smem_bytes<4>()));
  MGB_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<4, 1, true>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)tc_smem_bytes<4>()));
  MGB_CUDA(cudaFuncSetAttribute(tc_gemm_pkernel<false, kTcPBN, kTcPST, 2>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(TcPSmem<kTcPBN, kTcPST>) + 1024)));
  MGB_CUDA(cudaFuncSetAttribute(tc_gemm_pkernel<true, kTcPBN, kTcPST, 2>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(TcPSmem<kTcPBN, kTcPST>) + 1024)));
  MGB_CUDA(cudaMalloc(&g_tc_ctr, kTcCtrs * sizeof(int)));
  g_tc_ready = true;
  return 0;
}

static int make_map(CUtensorMap *m, const void *ptr, int bf16, int64_t rows,
                    int64_t k, int64_t ld, int box_rows) {
  cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kTcBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(
      m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16,
      2, const_cast<void *>(ptr), dims, strides, box, estr,
      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(MATGB_ERR_ARG, "tensor map encode failed (%d)", (int)r);
  return 0;
}

// C = beta*C + alpha*(*alpha_scale if given)*A*B^T.  A: M x K, B: N x K,
// K-contiguous 16-bit (bf16 != 0: BF16, else FP16); K a multiple of 64;
// lda, ldb multiples of 8 elements; 16-byte aligned bases.  With Alo and Blo
// (the remainders A - Ah, B - Bh, same layout) the three-product split form.
int tc_gemm(int bf16, int64_t M, int64_t N, int64_t K, const void *A,
            int64_t lda, const void *B, int64_t ldb, float alpha,
            const float *alpha_scale, float beta, float *C, int64_t ldc,
            int lower, const int32_t *skip, const void *Alo, const void *Blo,
            const float *rinv, const float *cinv, const void *Amid,
            const void *Bmid, int persist) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (M <= 0 || N <= 0) return 0;
  const bool split = Alo && Blo;
  const bool split3 = split && Amid && Bmid;
  const int nseg = split3 ? 6 : split ? 3 : 1;
  if (K <= 0 || K % kTcBK || (K / kTcBK) * nseg > kTcMaxKB || lda % 8 ||
      ldb % 8 || ((uintptr_t)A & 15) || ((uintptr_t)B & 15) ||
      ((uintptr_t)Alo & 15) || ((uintptr_t)Blo & 15) || ((uintptr_t)Amid & 15) ||
      ((uintptr_t)Bmid & 15) || M > INT32_MAX || N > INT32_MAX)
    return set_error(MATGB_ERR_ARG, "tc_gemm: unsupported shape/alignment");
  MGB_TRY(tc_setup());
  CUtensorMap ma, mb, mal, mbl, mam, mbm;
  MGB_TRY(make_map(&ma, A, bf16, M, K, lda, kTcBM));
  MGB_TRY(make_map(&mb, B, bf16, N, K, ldb, kTcBN));
  if (split) {
    MGB_TRY(make_map(&mal, Alo, bf16, M, K, lda, kTcBM));
    MGB_TRY(make_map(&mbl, Blo, bf16, N, K, ldb, kTcBN));
  } else {
    mal = ma;
    mbl = mb;
  }
  if (split3) {
    MGB_TRY(make_map(&mam, Amid, bf16, M, K, lda, kTcBM));
    MGB_TRY(make_map(&mbm, Bmid, bf16, N, K, ldb, kTcBN));
  } else {
    mam = ma;
    mbm = mb;
  }
  dim3 grid((unsigned)((M + kTcBM - 1) / kTcBM), (unsigned)((N + kTcBN - 1) / kTcBN));
  const uint32_t idesc = tc::idesc_f16(bf16 ? 1 : 0, kTcBM, kTcBN);
  const double frac = lower ? 0.5 : 1.0;
  // map per segment, 2 bits each (0 hi, 1 lo, 2 mid):
  //   split:  [Ah|Ah|Al] . [Bh|Bl|Bh]
  //   split3: [Ah|Ah|Am|Ah|Am|Al] . [Bh|Bm|Bh|Bl|Bm|Bh]  (the terms of weight
  //           1, 2^-11 and 2^-22; mid*lo, lo*mid and lo*lo are dropped)
  auto sel = [](std::initializer_list<unsigned> v) {
    unsigned m = 0, i = 0;
    for (unsigned x : v) m |= x << (2 * i++);
    return m;
  };
  const unsigned amask = split3 ? sel({0, 0, 2, 0, 2, 1}) : split ? sel({0, 0, 1}) : 0u;
  const unsigned bmask = split3 ? sel({0, 2, 0, 1, 2, 0}) : split ? sel({0, 1, 0}) : 0u;
  // long K (the plain GEMM): the deeper ring, one CTA per SM
  const bool deep = K * nseg > 32 * kTcBK;
  const char *nm = split3 ? (deep ? "tc_gemm_split3_k" : "tc_gemm_split3")
                   : deep   ? (split ? "tc_gemm_split_k" : "tc_gemm_k")
                            : (split ? "tc_gemm_split" : "tc_gemm");
  KtScope kt(nm, 2.0 * M * N * K * frac * nseg,
             4.0 * (beta != 0.f ? 2.0 : 1.0) * M * N * frac +
                 2.0 * (M + N) * K * (split3 ? 3 : split ? 2 : 1));
  if (rinv && !cinv)
    return set_error(MATGB_ERR_ARG, "tc_gemm: row scales need column scales");
  const bool sc = cinv != nullptr;  // rinv null: rows unscaled
#define MGB_TC_LAUNCH(ST_, MB_, SC_)                                           \
  tc_gemm_kernel<ST_, MB_, SC_><<<grid, kTcThreads, tc_smem_bytes<ST_>(),      \
                                  cx->stream>>>(                               \
      ma, mal, mam, mb, mbl, mbm, (int)M, (int)N, (int)(K / kTcBK), nseg,      \
      amask, bmask,                                                            \
      alpha, alpha_scale, beta, C, ldc, idesc, lower, skip, rinv, cinv, g_tc_err)
  const bool pers = persist < 0 ? g_tc_persistent != 0 : persist != 0;
  int *ctr = (!deep && pers) ? tile_counter(cx->stream) : nullptr;
  if (ctr) {
    CUtensorMap pb, pbl, pbm;  // B boxes of the persistent form's tile width
    MGB_TRY(make_map(&pb, B, bf16, N, K, ldb, kTcPBN));
    if (split) MGB_TRY(make_map(&pbl, Blo, bf16, N, K, ldb, kTcPBN)); else pbl = pb;
    if (split3) MGB_TRY(make_map(&pbm, Bmid, bf16, N, K, ldb, kTcPBN)); else pbm = pb;
    const int mt = (int)((M + kTcBM - 1) / kTcBM), nt = (int)((N + kTcPBN - 1) / kTcPBN);
    const int g = mt * nt < 2 * cx->sms ? mt * nt : 2 * cx->sms;
    const uint32_t pidesc = tc::idesc_f16(bf16 ? 1 : 0, kTcBM, kTcPBN);
    MGB_CUDA(cudaMemsetAsync(ctr, 0, sizeof(int), cx->stream));
#define MGB_TC_PLAUNCH(SC_)                                                        \
  tc_gemm_pkernel<SC_, kTcPBN, kTcPST, 2>                                          \
      <<<g, kTcThreads, sizeof(TcPSmem<kTcPBN, kTcPST>) + 1024, cx->stream>>>(     \
          ma, mal, mam, pb, pbl, pbm, (int)M, (int)N, (int)(K / kTcBK), nseg,      \
          amask, bmask, alpha, alpha_scale, beta, C, ldc, pidesc, lower, skip,     \
          rinv, cinv, g_tc_err, mt, nt, ctr)
    if (sc)
      MGB_TC_PLAUNCH(true);
    else
      MGB_TC_PLAUNCH(false);
#undef MGB_TC_PLAUNCH
  } else if (deep && sc)
    MGB_TC_LAUNCH(4, 1, true);
  else if (deep)
    MGB_TC_LAUNCH(4, 1, false);
  else if (sc)
    MGB_TC_LAUNCH(2, 2, true);
  else
    MGB_TC_LAUNCH(2, 2, false);
#undef MGB_TC_LAUNCH
  MGB_LAUNCHED("tc_gemm");
  return 0;
}

int tc_error_flag(int clear) {
  if (!g_tc_err) return 0;
  int h = 0;
  MGB_CUDA(cudaMemcpy(&h, g_tc_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (clear && h) MGB_CUDA(cudaMemset(g_tc_err, 0, sizeof(int)));
  return h;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_tc_gemm_dev(int bf16, size_t M, size_t N, size_t K, const void *A,
                      size_t lda, const void *B, size_t ldb, float alpha,
                      float beta, float *C, size_t ldc) {
  if (ldc < M) return set_error(MATGB_ERR_ARG, "tc_gemm: ldc < M");
  return tc_gemm(bf16, (int64_t)M, (int64_t)N, (int64_t)K, A, (int64_t)lda, B,
                 (int64_t)ldb, alpha, nullptr, beta, C, (int64_t)ldc, 0,
                 nullptr, nullptr, nullptr);
}

int matgb_tc_gemm_split_dev(size_t M, size_t N, size_t K, const void *Ah,
                            const void *Al, size_t lda, const void *Bh,
                            const void *Bl, size_t ldb, float alpha, float beta,
                            float *C, size_t ldc) {
  if (ldc < M) return set_error(MATGB_ERR_ARG, "tc_gemm_split: ldc < M");
  if (!Al || !Bl) return set_error(MATGB_ERR_ARG, "tc_gemm_split: null remainder");
  return tc_gemm(0, (int64_t)M, (int64_t)N, (int64_t)K, Ah, (int64_t)lda, Bh,
                 (int64_t)ldb, alpha, nullptr, beta, C, (int64_t)ldc, 0,
                 nullptr, Al, Bl);
}

int matgb_tc_persistent(int on) {
  const int prev = g_tc_persistent;
  if (on >= 0) g_tc_persistent = on ? 1 : 0;
  return prev;
}

int matgb_tc_status(void) {
  int f = tc_error_flag(1);
  if (f < 0) return f;
  return f ? set_error(MATGB_ERR_TIMEOUT,
                       "tensor-core kernel gave up waiting (flag %d)", f)
           : 0;
}

}  // extern "C"
