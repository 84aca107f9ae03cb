// The batched solver as ONE persistent launch (the default schedule; see
// batched.cu): every CTA first files a slice of the systems into the ten
// (size bucket, kind) queues, all CTAs meet at a grid barrier (the launch is
// cooperative, so every CTA is resident and the barrier cannot wait on a CTA
// that is not running; it is bounded all the same), then the CTAs drain the
// queues in five phases, largest systems first, with the register
// Gauss-Jordan solvers of batched_kernels.cuh:
//   orders 97..128: one system per CTA (128 threads);
//   orders 65..96:  one per CTA, 96 threads on a named barrier (the fourth
//                   warp waits for the next phase);
//   orders 33..64:  two per CTA, 64 threads each on a named barrier;
//   orders 17..32:  four per CTA, one warp each;
//   orders 1..16:   eight per CTA, one half warp each.
// (The double build solves orders 65..128 with the shared-memory rows of
// batched_smem.cuh, one system per CTA.)  Within a phase each group of threads
// pulls the next system from the phase's counter (general and SPD systems in
// one stream, general first), so the phases balance across the SMs by
// themselves; a CTA moves on when its groups find the phase empty.  Each
// system's status is first set to -4 (MATGB_ERR_TIMEOUT) and overwritten when
// it is solved: if the bounded grid barrier ever gave up, the unsolved
// systems say so.
#include "batched_smem.cuh"

namespace mgb {

constexpr int kFusedThreads = 128;
constexpr int kFusedPhases = 5;

struct FusedState {
  int count[kNumQueues];     // systems filed per queue
  int pnext[kFusedPhases];   // work counters per phase
  unsigned arrive;           // grid barrier arrivals
};

// One group's shared memory: a general or an SPD system (the groups of a
// phase run side by side, each on either kind, so each needs its own slot).
template <typename T, int NB>
union GroupSmem {
  BatchSmem<T, NB> lu;
  SpdSmem<T, NB> spd;
};

#ifdef MAT_DOUBLE_PRECISION
template <typename T>
union FusedSmem {
  SmemRows<T, 128> big;
  GroupSmem<T, 64> g64[2];
  GroupSmem<T, 32> g32[4];
  GroupSmem<T, 16> g16[8];
};
constexpr int kFusedMinB = 1;
#else
template <typename T>
union FusedSmem {
  GroupSmem<T, 128> g128;
  GroupSmem<T, 96> g96;
  GroupSmem<T, 64> g64[2];
  GroupSmem<T, 32> g32[4];
  GroupSmem<T, 16> g16[8];
};
constexpr int kFusedMinB = 3;  // the 128-row register frame: 170 registers
#endif

// Phase p's queues in the order they are drained (queue = 2*bucket + kind,
// general before SPD); the double build takes the 96 bucket in phase 0.
__device__ __forceinline__ int phase_nq(int p) {
#ifdef MAT_DOUBLE_PRECISION
  return p == 0 ? 4 : p == 1 ? 0 : 2;
#else
  return 2;
#endif
}
__device__ __forceinline__ int phase_queue(int p, int k) {
#ifdef MAT_DOUBLE_PRECISION
  if (p == 0) return k < 2 ? 8 + k : 4 + k;
#endif
  return 2 * (4 - p) + k;
}

template <typename T>
__global__ void __launch_bounds__(kFusedThreads, kFusedMinB)
    batched_fused_kernel(int64_t count, const int32_t *__restrict__ nvec,
                         const uint8_t *__restrict__ kind,
                         const int64_t *__restrict__ offA, const T *__restrict__ A,
                         const int64_t *__restrict__ offv, const T *__restrict__ b,
                         T *__restrict__ x, int32_t *__restrict__ status,
                         int32_t *__restrict__ list, FusedState *st, T eps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FusedSmem<T> &sm = *reinterpret_cast<FusedSmem<T> *>(smem_raw);
  __shared__ int take[8];
  __shared__ int qtot[kFusedPhases][4];  // queue sizes of each phase, in order
  __shared__ int gone;
  const int tid = threadIdx.x;
  // ---- file the systems into the queues: list[qi * count + pos]
  for (int64_t s = (int64_t)blockIdx.x * kFusedThreads + tid; s < count;
       s += (int64_t)gridDim.x * kFusedThreads) {
    const int n = nvec[s];
    if (n < 1 || n > 128) {
      status[s] = MATGB_ERR_ARG;  // -2: order not supported
      continue;
    }
    status[s] = MATGB_ERR_TIMEOUT;  // until solved
    const int qi = 2 * bucket_of(n) + (kind[s] == 1);
    const int pos = atomicAdd(&st->count[qi], 1);
    list[(int64_t)qi * count + pos] = (int32_t)s;
  }
  // ---- grid barrier: every CTA has filed its slice (the arrival is a
  // release after the CTA barrier, the wait an acquire before the next one)
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    atomicAdd(&st->arrive, 1u);
    const long long t0 = clock64();
    int ok = 1;
    for (int it = 0;; it++) {
      unsigned a;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(a) : "l"(&st->arrive) : "memory");
      if (a >= gridDim.x) break;
      if ((it & 63) == 63 && clock64() - t0 > (1ll << 31)) {  // ~1 s: give up
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    gone = !ok;
  }
  __syncthreads();
  if (gone) return;  // the systems not solved keep status -4
  if (tid < kFusedPhases * 4) {
    const int p = tid / 4, k = tid % 4;
    qtot[p][k] = k < phase_nq(p)
                     ? *reinterpret_cast<volatile int *>(&st->count[phase_queue(p, k)])
                     : 0;
  }
  __syncthreads();
  // item t of phase p -> queue qi, system s; false when the phase is empty
  auto item = [&](int p, int t, int &qi, int &s) -> bool {
    for (int k = 0; k < phase_nq(p); k++) {
      const int c = qtot[p][k];
      if (t < c) {
        qi = phase_queue(p, k);
        s = list[(int64_t)qi * count + t];
        return true;
      }
      t -= c;
    }
    return false;
  };
  // ---- phase 0: orders 97..128 (double: 65..128), one system per CTA
  for (;;) {
    if (tid == 0) take[0] = atomicAdd(&st->pnext[0], 1);
    __syncthreads();
    const int t = take[0];
    __syncthreads();
    int qi, s;
    if (!item(0, t, qi, s)) break;
    const int n = nvec[s];
    int r;
#ifdef MAT_DOUBLE_PRECISION
    if (qi & 1)
      r = solve_smem<T, 128, 1>(A + offA[s], n, b + offv[s], x + offv[s], sm.big, tid, eps);
    else
      r = solve_smem<T, 128, 0>(A + offA[s], n, b + offv[s], x + offv[s], sm.big, tid, eps);
#else
    if (qi & 1)
      r = solve_spd<T, 128>(A + offA[s], n, b + offv[s], x + offv[s], sm.g128.spd, tid);
    else
      r = solve_diag_first<T, 128>(A + offA[s], n, b + offv[s], x + offv[s], sm.g128.lu,
                                   tid, eps);
#endif
    if (tid == 0) status[s] = r;
    __syncthreads();
  }
  __syncthreads();
#ifndef MAT_DOUBLE_PRECISION
  // ---- phase 1: orders 65..96, one system per CTA on warps 0-2
  if (tid < 96) {
    const NamedBar bar{1, 96};
    for (;;) {
      if (tid == 0) take[0] = atomicAdd(&st->pnext[1], 1);
      bar();
      const int t = take[0];
      bar();
      int qi, s;
      if (!item(1, t, qi, s)) break;
      const int n = nvec[s];
      int r;
      if (qi & 1)
        r = solve_spd<T, 96>(A + offA[s], n, b + offv[s], x + offv[s], sm.g96.spd, tid, bar);
      else
        r = solve_diag_first<T, 96>(A + offA[s], n, b + offv[s], x + offv[s], sm.g96.lu,
                                    tid, eps, bar);
      if (tid == 0) status[s] = r;
      bar();
    }
  }
  __syncthreads();
#endif
  // ---- phase 2: orders 33..64, two groups of 64 threads
  {
    const int g = tid >> 6, i = tid & 63;
    const NamedBar bar{2 + g, 64};
    for (;;) {
      if (i == 0) take[g] = atomicAdd(&st->pnext[2], 1);
      bar();
      const int t = take[g];
      bar();
      int qi, s;
      if (!item(2, t, qi, s)) break;
      const int n = nvec[s];
      int r;
      if (qi & 1)
        r = solve_spd<T, 64>(A + offA[s], n, b + offv[s], x + offv[s], sm.g64[g].spd, i, bar);
      else
        r = solve_diag_first<T, 64>(A + offA[s], n, b + offv[s], x + offv[s], sm.g64[g].lu,
                                    i, eps, bar);
      if (i == 0) status[s] = r;
      bar();
    }
  }
  __syncthreads();
  // ---- phase 3: orders 17..32, a warp each
  {
    const int g = tid >> 5, i = tid & 31;
    for (;;) {
      if (i == 0) take[g] = atomicAdd(&st->pnext[3], 1);
      __syncwarp();
      const int t = take[g];
      __syncwarp();
      int qi, s;
      if (!item(3, t, qi, s)) break;
      const int n = nvec[s];
      int r;
      if (qi & 1)
        r = solve_spd<T, 32>(A + offA[s], n, b + offv[s], x + offv[s], sm.g32[g].spd, i);
      else
        r = solve_diag_first<T, 32>(A + offA[s], n, b + offv[s], x + offv[s], sm.g32[g].lu,
                                    i, eps);
      if (i == 0) status[s] = r;
      __syncwarp();
    }
  }
  __syncthreads();
  // ---- phase 4: orders 1..16, a half warp each
  {
    const int g = tid >> 4, i = tid & 15;
    const unsigned gm = 0xffffu << (tid & 16);
    for (;;) {
      if (i == 0) take[g] = atomicAdd(&st->pnext[4], 1);
      __syncwarp(gm);
      const int t = take[g];
      __syncwarp(gm);
      int qi, s;
      if (!item(4, t, qi, s)) break;
      const int n = nvec[s];
      int r;
      if (qi & 1)
        r = solve_spd<T, 16>(A + offA[s], n, b + offv[s], x + offv[s], sm.g16[g].spd, i);
      else
        r = solve_diag_first<T, 16>(A + offA[s], n, b + offv[s], x + offv[s], sm.g16[g].lu,
                                    i, eps);
      if (i == 0) status[s] = r;
      __syncwarp(gm);
    }
  }
}

static size_t fused_smem_bytes() { return sizeof(FusedSmem<elem_t>); }
static int g_fused_per_sm[65] = {};  // occupancy by cap (0: none), per process

// Shared-memory attribute and occupancy, once (kept out of stream capture).
int fused_prepare(int ctas_per_sm) {
  auto k = batched_fused_kernel<elem_t>;
  const size_t smem = fused_smem_bytes();
  if (ctas_per_sm < 0 || ctas_per_sm > 64) ctas_per_sm = 0;
  if (g_fused_per_sm[ctas_per_sm] > 0) return 0;
  MGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
  int per_sm = 0;
  MGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kFusedThreads, smem));
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  if (per_sm < 1) return set_error(MATGB_ERR_CUDA, "batched: fused kernel does not fit an SM");
  g_fused_per_sm[ctas_per_sm] = per_sm;
  return 0;
}

int launch_fused(int64_t count, const int32_t *n, const int64_t *offA,
                 const elem_t *A, const int64_t *offv, const elem_t *b, elem_t *x,
                 const uint8_t *kind, int32_t *status, int32_t *list,
                 void *state, int ctas_per_sm) {
  auto k = batched_fused_kernel<elem_t>;
  const size_t smem = fused_smem_bytes();
  if (ctas_per_sm < 0 || ctas_per_sm > 64) ctas_per_sm = 0;
  MGB_TRY(fused_prepare(ctas_per_sm));
  const int per_sm = g_fused_per_sm[ctas_per_sm];
  FusedState *st = reinterpret_cast<FusedState *>(state);
  elem_t eps = kPivotEps;
  void *args[] = {(void *)&count, (void *)&n,      (void *)&kind, (void *)&offA,
                  (void *)&A,     (void *)&offv,   (void *)&b,    (void *)&x,
                  (void *)&status, (void *)&list,  (void *)&st,   (void *)&eps};
  MGB_CUDA(cudaMemsetAsync(st, 0, sizeof(FusedState), ctx()->stream));
  KtScope kt("batched_fused", 0.0, 0.0);
  MGB_CUDA(cudaLaunchCooperativeKernel((const void *)k, dim3(ctx()->sms * per_sm),
                                       dim3(kFusedThreads), args, smem, ctx()->stream));
  MGB_LAUNCHED("batched_fused");
  return 0;
}

size_t fused_state_bytes() { return sizeof(FusedState); }

}  // namespace mgb
