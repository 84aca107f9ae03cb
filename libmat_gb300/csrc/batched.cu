// Batched solves of many small, uneven systems in one pass: the GB300 form of
// calling mat_solve (mat.h:4807-4837) / mat_solve_spd (mat.h:4839-4871) in a
// loop over independent systems.
//
// Layout: all matrices packed back to back in one buffer (system s at
// A + offA[s], column-major, leading dimension n_s), right-hand sides and
// solutions packed at offv[s].  kind[s] = 0 solves a general system with the
// reference's partial-pivoting rule (first index of max |a|, tiny pivots
// swapped in but not eliminated with), kind[s] = 1 an SPD system (status -1
// when a pivot is <= 0, as mat_solve_spd returns -1; x is then left
// untouched).
//
// Kernel: one thread per matrix row, the row (and its right-hand-side entry)
// held in registers, one system per group of NB threads, NB a compile-time
// size bucket (16, 32, 64, 96, 128; two 16-row systems share a warp); the
// double build covers orders up to 64.  Gauss-Jordan elimination in a
// shifted register frame (the pivot column is always register 0, so the step
// loop is an ordinary loop over statically indexed registers): one barrier
// per step, the pivot chosen by warp shuffles then across warps through
// shared memory, the winning row read by every row from its warp's slot,
// rows above the pivot eliminated too so no back substitution is needed.
// General systems use partial pivoting with mat_plu's pivot rule (rows trade
// roles, not data); SPD systems rebuild the symmetric matrix from the lower
// triangle (what mat_chol reads), do no exchanges and report -1 when a
// pivot -- the Schur-complement diagonal mat_chol tests -- is <= 0.
//
// Scheduling: a device-side pre-pass sorts systems into (size bucket, kind)
// queues; one persistent launch per queue pulls systems with an atomic
// counter, largest sizes first.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <string>

#include "batched_kernels.cuh"

namespace mgb {

// ---- schedule table -----------------------------------------------------------
// Compiled-in defaults: the register Gauss-Jordan kernels everywhere (the
// blocked LU measured 2.5-3x slower on the 100k-system workload: its panel,
// one warp's serial chain of 8 columns, idles the CTA), occupancy as the
// kernels' resources allow.  tune_batched.py measures the alternatives on the
// device and writes libmat_gb300/batched_tune.json (or
// $LIBMATGB_BATCHED_TUNE), read once at the first batched call; entries it
// does not name keep their defaults.
static BatchTune g_tune[kNumBuckets][2] = {
    {{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}, {{0, 0}, {0, 0}},
    {{0, 0}, {0, 0}}};
// The launch-per-queue schedule is the compiled default: on the 100k-system
// workload the one-launch kernel took 5.58 ms against 4.69 ms for the queue
// launches (its shared register budget holds the 65..96 phase to 3 systems
// per SM where that queue's own kernel keeps 4, and its 128-row frame
// spills).  Both are replayed as CUDA graphs; the tuner's file may choose.
static int g_fused = 0;       // 1: one persistent launch; 0: a launch per queue
static int g_fused_ctas = 0;  // resident CTAs per SM for it (0: as many as fit)
static int g_graphs = 1;      // replay the launch sequence as a CUDA graph
// The mixed-precision mode (float build): 0 off; 1 the queues of orders
// 33..128 whose entry below is 1 take the tensor-core kernels (batched_tc.cu),
// refined to an FP32-level residual, the others keep the FP32 kernels; 2 every
// queue of orders 33..128 takes them.  Compiled-in: the 97..128 general queue
// only -- measured on the 100k-system workload, the tensor-core kernel took
// 1.20 ms there against 1.59 ms for the register kernel, and lost on the
// other queues (SPD 97..128: 1.55 against 1.21 ms).  The tuner's file
// ("mixed_tc" entries) may choose.
static int g_mixed = 0;
static int g_mixed_tc[kNumBuckets][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {1, 0}};
static bool g_graphs_broken = false;
static std::once_flag g_tune_once;
static char g_tune_source[512] = "defaults";

// Reads {"entries": [{"prec": "f32", "nb": 128, "kind": 0, "algo": 1,
// "ctas_per_sm": 2}, ...]} -- a flat list of objects; each needs nb, kind,
// algo and ctas_per_sm, and one whose "prec" names the other build is
// skipped.  (Other keys, and other objects without those keys, are
// ignored.)
static int int_after(const char *p, const char *key, const char *end, int *out) {
  const char *k = strstr(p, key);
  if (!k || k >= end) return 0;
  k = strchr(k + strlen(key), ':');
  if (!k || k >= end) return 0;
  return sscanf(k + 1, "%d", out) == 1;
}

static void load_tune_file() {
  const char *env = getenv("LIBMATGB_BATCHED_TUNE");
  std::string path;
  if (env && *env) {
    path = env;
  } else {
    // next to the package: <lib dir>/../batched_tune.json
    const char *libdir = matgb_library_dir();
    if (!libdir || !*libdir) return;
    path = std::string(libdir) + "/../batched_tune.json";
  }
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return;
  std::string text;
  char buf[4096];
  size_t got;
  while ((got = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
  fclose(f);
  int used = 0;
  {
    // top-level schedule keys (before the entries list)
    const char *t = text.c_str();
    const char *lst = strstr(t, "\"entries\"");
    const char *end = lst ? lst : t + text.size();
    int v;
    if (int_after(t, "\"fused\"", end, &v) && (v == 0 || v == 1)) g_fused = v;
    if (int_after(t, "\"fused_ctas_per_sm\"", end, &v) && v >= 0 && v <= 64)
      g_fused_ctas = v;
  }
  for (const char *p = strchr(text.c_str(), '{'); p; ) {
    p = strchr(p + 1, '{');
    if (!p) break;
    const char *e = strchr(p, '}');
    if (!e) break;
    // entries for the other precision's library are skipped
    const char *pk = strstr(p, "\"prec\"");
    if (pk && pk < e) {
      const char *want = sizeof(elem_t) == 8 ? "f64" : "f32";
      const char *v = strchr(pk + 6, '"');
      if (!v || v >= e || strncmp(v + 1, want, 3) != 0) {
        p = e;
        continue;
      }
    }
    int nb, kind, algo, ctas, mtc;
    if (sizeof(elem_t) == 4 && int_after(p, "\"nb\"", e, &nb) &&
        int_after(p, "\"kind\"", e, &kind) && int_after(p, "\"mixed_tc\"", e, &mtc) &&
        (kind == 0 || kind == 1) && (mtc == 0 || mtc == 1)) {
      for (int bk = 2; bk < kNumBuckets; bk++)
        if (bucket_nb(bk) == nb) {
          g_mixed_tc[bk][kind] = mtc;
          used++;
        }
      p = e;
      continue;
    }
    if (int_after(p, "\"nb\"", e, &nb) && int_after(p, "\"kind\"", e, &kind) &&
        int_after(p, "\"algo\"", e, &algo) &&
        int_after(p, "\"ctas_per_sm\"", e, &ctas) && (kind == 0 || kind == 1) &&
        (algo == 0 || algo == 1) && ctas >= 0 && ctas <= 64) {
      for (int bk = 0; bk < kNumBuckets; bk++)
        if (bucket_nb(bk) == nb && (algo == 0 || nb >= 64)) {
          g_tune[bk][kind] = BatchTune{algo, ctas};
          used++;
        }
    }
    p = e;
  }
  snprintf(g_tune_source, sizeof g_tune_source, "%s (%d entries)", path.c_str(), used);
}

const BatchTune &batched_tune(int bucket, int kind) {
  std::call_once(g_tune_once, load_tune_file);
  return g_tune[bucket][kind ? 1 : 0];
}

// queue = 2*bucket + kind; counts per queue, then the list is grouped by queue
__global__ void bucket_count_kernel(int64_t count, const int32_t *__restrict__ n,
                                    const uint8_t *__restrict__ kind,
                                    BatchQueues *q) {
  __shared__ int h[kNumQueues];
  if (threadIdx.x < kNumQueues) h[threadIdx.x] = 0;
  __syncthreads();
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < count;
       s += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&h[2 * bucket_of(n[s]) + (kind[s] == 1)], 1);
  __syncthreads();
  if (threadIdx.x < kNumQueues) atomicAdd(&q->count[threadIdx.x], h[threadIdx.x]);
}

__global__ void bucket_scatter_kernel(int64_t count,
                                      const int32_t *__restrict__ n,
                                      const uint8_t *__restrict__ kind,
                                      BatchQueues *q, int32_t *__restrict__ list) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < count;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int qi = 2 * bucket_of(n[s]) + (kind[s] == 1);
    int base = 0;
    for (int i = 0; i < qi; i++) base += q->count[i];
    const int pos = atomicAdd(&q->fill[qi], 1);
    list[base + pos] = (int32_t)s;
  }
}

// Orders outside what this build supports get status -2 and are not solved
// (1..128 in float, 1..64 in double).
__global__ void check_sizes_kernel(int64_t count, const int32_t *__restrict__ n,
                                   int nmax, int32_t *__restrict__ status) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < count;
       s += (int64_t)gridDim.x * blockDim.x)
    if (n[s] < 1 || n[s] > nmax) status[s] = -2;
}

// ---- the one-launch schedule (batched_fused.cu), replayed as a CUDA graph -----
int launch_fused(int64_t count, const int32_t *n, const int64_t *offA,
                 const elem_t *A, const int64_t *offv, const elem_t *b, elem_t *x,
                 const uint8_t *kind, int32_t *status, int32_t *list, void *state,
                 int ctas_per_sm);
int fused_prepare(int ctas_per_sm);
size_t fused_state_bytes();


// The graph of the last call's arguments: the launch sequence of either
// schedule (the memset of the queue state and the cooperative launch; or the
// memset, two filing kernels, the ten queue launches and the size check),
// captured once and replayed while the caller passes the same buffers (the
// usual case: a solver called again on new data in the same buffers) and the
// schedule is unchanged.
struct GraphKey {
  int64_t count;
  const void *p[11];
  int fused, ctas, version;
  bool operator==(const GraphKey &o) const {
    if (count != o.count || fused != o.fused || ctas != o.ctas || version != o.version)
      return false;
    for (int i = 0; i < 11; i++)
      if (p[i] != o.p[i]) return false;
    return true;
  }
};
static GraphKey g_gkey{};
static BatchQueues *g_last_q = nullptr;  // the last queue-schedule call's state
static cudaGraphExec_t g_gexec = nullptr;
static int g_tune_version = 0;  // bumped by matgb_batched_tune / _schedule
static int g_graph_kernels = 0;

template <class F>
static int run_graph(const GraphKey &key, F enqueue) {
  cudaStream_t st = ctx()->stream;
  if (!g_graphs || g_graphs_broken || ktime_on()) return enqueue();
  if (!(g_gexec && key == g_gkey)) {
    if (g_gexec) {
      cudaGraphExecDestroy(g_gexec);
      g_gexec = nullptr;
    }
    const unsigned long long before = launch_counter();
    cudaGraph_t graph = nullptr;
    // relaxed: the queue launchers' occupancy queries run inside the capture
    MGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    const int r = enqueue();
    const cudaError_t e = cudaStreamEndCapture(st, &graph);
    g_graph_kernels = (int)(launch_counter() - before);
    launch_counter_set(before);
    if (r != 0 || e != cudaSuccess || !graph ||
        cudaGraphInstantiate(&g_gexec, graph, 0) != cudaSuccess) {
      // capture of this sequence is not supported here: launch directly
      // from now on
      if (graph) cudaGraphDestroy(graph);
      g_gexec = nullptr;
      cudaGetLastError();
      matgb_clear_error();
      g_graphs_broken = true;
      return enqueue();
    }
    cudaGraphDestroy(graph);
    g_gkey = key;
  }
  MGB_CUDA(cudaGraphLaunch(g_gexec, st));
  launch_counter_set(launch_counter() + (unsigned long long)g_graph_kernels);
  return 0;
}

static int solve_fused(int64_t count, const int32_t *n, const int64_t *offA,
                       const elem_t *A, const int64_t *offv, const elem_t *b,
                       elem_t *x, const uint8_t *kind, int32_t *status) {
  cudaStream_t st = ctx()->stream;
  int32_t *list = (int32_t *)ws(WS_V1, (size_t)kNumQueues * count * sizeof(int32_t));
  void *state = ws(WS_T2, fused_state_bytes() + 256);
  if (!list || !state) return MATGB_ERR_NOMEM;
  MGB_TRY(fused_prepare(g_fused_ctas));  // attributes, occupancy (not captured)
  const GraphKey key{count, {n, offA, A, offv, b, x, kind, status, list, state, st},
                     1, g_fused_ctas, g_tune_version};
  return run_graph(key, [&] {
    return launch_fused(count, n, offA, A, offv, b, x, kind, status, list, state,
                        g_fused_ctas);
  });
}

static int enqueue_queues(int64_t count, const int32_t *n, const int64_t *offA,
                          const elem_t *A, const int64_t *offv, const elem_t *b,
                          elem_t *x, const uint8_t *kind, int32_t *status,
                          BatchQueues *q, int32_t *list) {
  cudaStream_t st = ctx()->stream;
  MGB_CUDA(cudaMemsetAsync(q, 0, sizeof(BatchQueues) + sizeof(int), st));
  const unsigned g = (unsigned)((count + 255) / 256 < 1024 ? (count + 255) / 256 : 1024);
  constexpr int nmax = 128;
  bucket_count_kernel<<<g, 256, 0, st>>>(count, n, kind, q);
  MGB_LAUNCHED("bucket_count");
  bucket_scatter_kernel<<<g, 256, 0, st>>>(count, n, kind, q, list);
  MGB_LAUNCHED("bucket_scatter");
  // the largest systems first, so the long ones start early
  for (int bk = kNumBuckets - 1; bk >= 0; bk--)
    for (int kd = 0; kd < 2; kd++) {
      const int qi = 2 * bk + kd;
      using Fn = int (*)(int, const int32_t *, BatchQueues *, const int32_t *,
                         const int64_t *, const elem_t *, const int64_t *,
                         const elem_t *, elem_t *, int32_t *);
      static const Fn fns[kNumBuckets][2] = {
          {batched_bucket_16_lu, batched_bucket_16_chol},
          {batched_bucket_32_lu, batched_bucket_32_chol},
          {batched_bucket_64_lu, batched_bucket_64_chol},
          {batched_bucket_96_lu, batched_bucket_96_chol},
          {batched_bucket_128_lu, batched_bucket_128_chol}};
      if ((g_mixed == 2 && bk >= 2) || (g_mixed == 1 && g_mixed_tc[bk][kd]))
        MGB_TRY(batched_tc_bucket(bk, kd, qi, list, q, n, offA, A, offv, b, x, status,
                                  0));
      else
        MGB_TRY(fns[bk][kd](qi, list, q, n, offA, A, offv, b, x, status));
    }
  check_sizes_kernel<<<g, 256, 0, st>>>(count, n, nmax, status);
  MGB_LAUNCHED("check_sizes");
  return 0;
}

int solve_batched(int64_t count, const int32_t *n, const int64_t *offA,
                  const elem_t *A, const int64_t *offv, const elem_t *b,
                  elem_t *x, const uint8_t *kind, int32_t *status) {
  Ctx *cx = ctx();
  if (!cx) return MATGB_ERR_NO_DEVICE;
  if (count <= 0) return 0;
  if (count > INT32_MAX / kNumQueues) return set_error(MATGB_ERR_ARG, "batch too large");
  (void)batched_tune(0, 0);  // the schedule table, loaded once
  // the one-launch schedule has no mixed-precision phases
  if (g_fused && !g_mixed) return solve_fused(count, n, offA, A, offv, b, x, kind, status);
  BatchQueues *q = (BatchQueues *)ws(WS_T2, sizeof(BatchQueues) + 256);
  int32_t *list = (int32_t *)ws(WS_V1, (size_t)count * sizeof(int32_t));
  if (!q || !list) return MATGB_ERR_NOMEM;
  g_last_q = q;
  const GraphKey key{count, {n, offA, A, offv, b, x, kind, status, list, q, cx->stream},
                     0, g_mixed, g_tune_version};
  return run_graph(key, [&] {
    return enqueue_queues(count, n, offA, A, offv, b, x, kind, status, q, list);
  });
}

}  // namespace mgb

using namespace mgb;

extern "C" int matgb_batched_tune(int nb, int kind, int algo, int ctas_per_sm) {
  (void)batched_tune(0, 0);  // the file (if any) is read first, then overridden
  if ((kind != 0 && kind != 1) || (algo != 0 && algo != 1) || ctas_per_sm < 0 ||
      ctas_per_sm > 64)
    return set_error(MATGB_ERR_ARG, "batched_tune: bad kind/algo/ctas_per_sm");
  for (int bk = 0; bk < kNumBuckets; bk++)
    if (bucket_nb(bk) == nb) {
      if (algo == 1 && nb < 64)
        return set_error(MATGB_ERR_ARG, "batched_tune: blocked form needs nb >= 64");
      g_tune[bk][kind] = BatchTune{algo, ctas_per_sm};
      g_tune_version++;
      return 0;
    }
  return set_error(MATGB_ERR_ARG, "batched_tune: nb must be 16, 32, 64, 96 or 128");
}

extern "C" int matgb_batched_tune_get(int nb, int kind, int *algo, int *ctas_per_sm) {
  for (int bk = 0; bk < kNumBuckets; bk++)
    if (bucket_nb(bk) == nb && (kind == 0 || kind == 1)) {
      const BatchTune &t = batched_tune(bk, kind);
      if (algo) *algo = t.algo;
      if (ctas_per_sm) *ctas_per_sm = t.ctas_per_sm;
      return 0;
    }
  return set_error(MATGB_ERR_ARG, "batched_tune_get: bad nb/kind");
}

extern "C" int matgb_batched_schedule(int fused, int ctas_per_sm, int graphs) {
  (void)batched_tune(0, 0);
  const int prev = g_fused;
  if (fused >= 0) g_fused = fused ? 1 : 0;
  if (ctas_per_sm >= 0) g_fused_ctas = ctas_per_sm;
  if (graphs >= 0) g_graphs = graphs ? 1 : 0;
  g_tune_version++;
  return prev;
}

extern "C" int matgb_batched_mixed(int on) {
  (void)batched_tune(0, 0);  // the file's entries first
  const int prev = g_mixed;
  if (on >= 0) {
    if (on > 2) return set_error(MATGB_ERR_ARG, "batched_mixed: on must be 0, 1 or 2");
#ifdef MAT_DOUBLE_PRECISION
    if (on) return set_error(MATGB_ERR_ARG, "the mixed batched solver is float-only");
#endif
    g_mixed = on;
    g_tune_version++;
  }
  return prev;
}

extern "C" int matgb_batched_mixed_tune(int nb, int kind, int use_tc) {
  (void)batched_tune(0, 0);
  if ((kind != 0 && kind != 1) || (use_tc != 0 && use_tc != 1))
    return set_error(MATGB_ERR_ARG, "batched_mixed_tune: bad kind/use_tc");
  for (int bk = 2; bk < kNumBuckets; bk++)
    if (bucket_nb(bk) == nb) {
      g_mixed_tc[bk][kind] = use_tc;
      g_tune_version++;
      return 0;
    }
  return set_error(MATGB_ERR_ARG, "batched_mixed_tune: nb must be 64, 96 or 128");
}

extern "C" int matgb_batched_mixed_stats(int *corrections, int *unconverged, int *timeouts) {
  int h[3] = {0, 0, 0};
  if (g_last_q) {
    Ctx *cx = ctx();
    if (!cx) return MATGB_ERR_NO_DEVICE;
    MGB_CUDA(cudaStreamSynchronize(cx->stream));
    MGB_CUDA(cudaMemcpy(h, &g_last_q->tc_corr, sizeof h, cudaMemcpyDeviceToHost));
  }
  if (corrections) *corrections = h[0];
  if (unconverged) *unconverged = h[1];
  if (timeouts) *timeouts = h[2];
  return 0;
}

extern "C" const char *matgb_batched_tune_source(void) {
  (void)batched_tune(0, 0);
  return g_tune_source;
}

extern "C" int matgb_solve_batched_dev(int64_t count, const int32_t *n,
                                       const int64_t *offA, const mat_elem_t *A,
                                       const int64_t *offv, const mat_elem_t *b,
                                       mat_elem_t *x, const uint8_t *kind,
                                       int32_t *status) {
  return solve_batched(count, n, offA, A, offv, b, x, kind, status);
}
