// Runtime: device context, library stream, error channel, grow-only device
// workspace, events, memory helpers and seeded device-side input generation.
#include <dlfcn.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "internal.cuh"

namespace mgb {

static Ctx g_ctx;
static std::mutex g_mu;
static char g_err[1024];
static int g_abort_on_error = 1;
static std::atomic<unsigned long long> g_launches{0};

struct WsBuf {
  void *p = nullptr;
  size_t cap = 0;
};
static WsBuf g_ws[WS_NSLOTS];

static int init_locked(int device) {
  if (g_ctx.device >= 0) return 0;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return set_error(MATGB_ERR_NO_DEVICE, "no CUDA device visible (%s)",
                     cudaGetErrorString(e));
  if (device < 0 || device >= count)
    return set_error(MATGB_ERR_ARG, "device %d out of range", device);
  MGB_CUDA(cudaSetDevice(device));
  MGB_CUDA(cudaDeviceGetAttribute(&g_ctx.sms, cudaDevAttrMultiProcessorCount,
                                  device));
  MGB_CUDA(cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking));
  for (int i = 0; i < 16; i++) MGB_CUDA(cudaEventCreate(&g_ctx.ev[i]));
  g_ctx.device = device;
  return 0;
}

Ctx *ctx() {
  if (g_ctx.device < 0) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (init_locked(0) != 0) return nullptr;
  }
  return &g_ctx;
}

int set_error(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
  cudaGetLastError();  // do not let a returned error resurface at a later check
  return set_error(MATGB_ERR_CUDA, "%s failed: %s (%s:%d)", what,
                   cudaGetErrorString(e), file, line);
}

void fail_void(const char *where) {
  fprintf(stderr, "libmatgb: %s: %s\n", where, g_err);
  if (g_abort_on_error) abort();
}

// As launched(), and on failure the message carries the kernel's registered
// limits next to the dynamic shared memory the launch asked for.
int launch_check(const void *func, const char *name, size_t smem) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return 0;
  cudaFuncAttributes fa{};
  cudaError_t e2 = cudaFuncGetAttributes(&fa, func);
  cudaGetLastError();
  return set_error(MATGB_ERR_CUDA,
                   "launch of %s failed: %s (dynamic smem asked %zu, kernel max "
                   "dynamic %d, static %zu, regs %d, attr query %s)",
                   name, cudaGetErrorString(e), smem, fa.maxDynamicSharedSizeBytes,
                   fa.sharedSizeBytes, fa.numRegs, cudaGetErrorString(e2));
}

unsigned long long launch_counter() { return g_launches.load(); }
void launch_counter_set(unsigned long long v) { g_launches.store(v); }

int launched(const char *name) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return set_error(MATGB_ERR_CUDA, "launch of %s failed: %s", name,
                     cudaGetErrorString(e));
  return 0;
}

void *ws(int slot, size_t bytes) {
  if (slot < 0 || slot >= WS_NSLOTS) return nullptr;
  if (bytes == 0) bytes = 256;
  WsBuf &b = g_ws[slot];
  if (b.cap >= bytes) return b.p;
  if (b.p) {
    // The buffer may still be in use by queued work.
    cudaStreamSynchronize(g_ctx.stream);
    cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
  }
  size_t cap = (bytes + 0xFFFFF) & ~(size_t)0xFFFFF;  // 1 MiB granules
  cudaError_t e = cudaMalloc(&b.p, cap);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(MATGB_ERR_NOMEM, "device workspace of %zu bytes: %s", cap,
              cudaGetErrorString(e));
    b.p = nullptr;
    return nullptr;
  }
  b.cap = cap;
  return b.p;
}

// ---- seeded generation ------------------------------------------------------
// splitmix64 finaliser over (seed, index): u = top 53 bits / 2^53 in [0,1).
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(uint64_t seed, uint64_t i) {
  return (double)(splitmix64(seed * 0x100000001B3ull + i) >> 11) *
         (1.0 / 9007199254740992.0);
}

__global__ void fill_uniform_kernel(elem_t *A, size_t count, uint64_t seed,
                                    double lo, double hi) {
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += stride)
    A[i] = (elem_t)(lo + (hi - lo) * u01(seed, i));
}

// Box-Muller on the pair (2*(i/2), 2*(i/2)+1): even i takes the cosine
// branch, odd i the sine branch.  u1 is shifted into (0,1] so log is finite.
__global__ void fill_normal_kernel(elem_t *A, size_t count, uint64_t seed) {
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += stride) {
    size_t p = i & ~(size_t)1;
    double u1 = 1.0 - u01(seed, p);
    double u2 = u01(seed, p + 1);
    double r = sqrt(-2.0 * log(u1));
    double t = 6.283185307179586 * u2;
    A[i] = (elem_t)((i & 1) ? r * sin(t) : r * cos(t));
  }
}

__global__ void add_diag_kernel(elem_t *A, size_t n, size_t lda,
                                double shift) {
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += stride)
    A[i * lda + i] = (elem_t)((double)A[i * lda + i] + shift);
}

static int grid_for(size_t count) {
  Ctx *c = ctx();
  size_t g = (count + 255) / 256;
  size_t cap = (size_t)(c ? c->sms : 148) * 8;
  if (g > cap) g = cap;
  if (g == 0) g = 1;
  return (int)g;
}

}  // namespace mgb

using namespace mgb;

extern "C" {

int matgb_init(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_ctx.device >= 0)
    return g_ctx.device == device
               ? 0
               : set_error(MATGB_ERR_ARG, "already initialised on device %d",
                           g_ctx.device);
  return init_locked(device);
}

int matgb_elem_size(void) { return (int)sizeof(elem_t); }

const char *matgb_last_error(void) { return g_err; }
void matgb_clear_error(void) { g_err[0] = 0; }
void matgb_set_abort_on_error(int on) { g_abort_on_error = on; }

int matgb_sync(void) {
  Ctx *c = ctx();
  if (!c) return MATGB_ERR_NO_DEVICE;
  MGB_CUDA(cudaStreamSynchronize(c->stream));
  return 0;
}

void *matgb_stream(void) {
  Ctx *c = ctx();
  return c ? (void *)c->stream : nullptr;
}

unsigned long long matgb_launch_count(void) { return g_launches.load(); }

int matgb_sm_count(void) {
  Ctx *c = ctx();
  return c ? c->sms : 0;
}

const char *matgb_library_dir(void) {
  static char dir[1024];
  static std::once_flag once;
  std::call_once(once, [] {
    Dl_info info;
    dir[0] = 0;
    if (dladdr(reinterpret_cast<void *>(&matgb_library_dir), &info) && info.dli_fname) {
      strncpy(dir, info.dli_fname, sizeof dir - 1);
      dir[sizeof dir - 1] = 0;
      char *slash = strrchr(dir, '/');
      if (slash)
        *slash = 0;
      else
        strcpy(dir, ".");
    }
  });
  return dir;
}

void *matgb_device_alloc(size_t bytes) {
  if (!ctx()) return nullptr;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(MATGB_ERR_NOMEM, "cudaMalloc(%zu): %s", bytes,
              cudaGetErrorString(e));
    return nullptr;
  }
  return p;
}

int matgb_device_free(void *p) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  MGB_CUDA(cudaFree(p));
  return 0;
}

void *matgb_host_alloc(size_t bytes) {
  if (!ctx()) return nullptr;
  void *p = nullptr;
  cudaError_t e = cudaMallocHost(&p, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(MATGB_ERR_NOMEM, "cudaMallocHost(%zu): %s", bytes,
              cudaGetErrorString(e));
    return nullptr;
  }
  return p;
}

int matgb_host_free(void *p) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  MGB_CUDA(cudaFreeHost(p));
  return 0;
}

static int copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind k) {
  Ctx *c = ctx();
  if (!c) return MATGB_ERR_NO_DEVICE;
  if (bytes == 0) return 0;
  MGB_CUDA(cudaMemcpyAsync(dst, src, bytes, k, c->stream));
  return 0;
}

int matgb_memcpy_h2d(void *dst, const void *src, size_t bytes) {
  return copy(dst, src, bytes, cudaMemcpyHostToDevice);
}
int matgb_memcpy_d2h(void *dst, const void *src, size_t bytes) {
  return copy(dst, src, bytes, cudaMemcpyDeviceToHost);
}
int matgb_memcpy_d2d(void *dst, const void *src, size_t bytes) {
  return copy(dst, src, bytes, cudaMemcpyDeviceToDevice);
}
int matgb_memset_dev(void *dst, int value, size_t bytes) {
  Ctx *c = ctx();
  if (!c) return MATGB_ERR_NO_DEVICE;
  MGB_CUDA(cudaMemsetAsync(dst, value, bytes, c->stream));
  return 0;
}

int matgb_event_record(int slot) {
  Ctx *c = ctx();
  if (!c) return MATGB_ERR_NO_DEVICE;
  if (slot < 0 || slot >= 16) return set_error(MATGB_ERR_ARG, "event slot");
  MGB_CUDA(cudaEventRecord(c->ev[slot], c->stream));
  return 0;
}

double matgb_event_elapsed_ms(int slot0, int slot1) {
  Ctx *c = ctx();
  if (!c || slot0 < 0 || slot0 >= 16 || slot1 < 0 || slot1 >= 16) return -1.0;
  if (cudaEventSynchronize(c->ev[slot1]) != cudaSuccess) return -1.0;
  float ms = -1.f;
  if (cudaEventElapsedTime(&ms, c->ev[slot0], c->ev[slot1]) != cudaSuccess)
    return -1.0;
  return (double)ms;
}

int matgb_fill_uniform_dev(mat_elem_t *A, size_t count, uint64_t seed,
                           double lo, double hi) {
  Ctx *c = ctx();
  if (!c) return MATGB_ERR_NO_DEVICE;
  if (count == 0) return 0;
  fill_uniform_kernel<<<grid_for(count), 256, 0, c->stream>>>(A, count, seed,
                                                              lo, hi);
  MGB_LAUNCHED("fill_uniform");
  return 0;
}

int matgb_fill_normal_dev(mat_elem_t *A, size_t count, uint64_t seed) {
  Ctx *c = ctx();
  if (!c) return MATGB_ERR_NO_DEVICE;
  if (count == 0) return 0;
  fill_normal_kernel<<<grid_for(count), 256, 0, c->stream>>>(A, count, seed);
  MGB_LAUNCHED("fill_normal");
  return 0;
}

int matgb_add_diag_dev(mat_elem_t *A, size_t n, size_t lda, double shift) {
  Ctx *c = ctx();
  if (!c) return MATGB_ERR_NO_DEVICE;
  if (n == 0) return 0;
  add_diag_kernel<<<grid_for(n), 256, 0, c->stream>>>(A, n, lda, shift);
  MGB_LAUNCHED("add_diag");
  return 0;
}

}  // extern "C"

// ---- per-kernel timing ------------------------------------------------------
#include <string>
#include <vector>

namespace mgb {

struct KtRec {
  std::string name;
  cudaEvent_t a, b;
  double flops, bytes;
  cudaStream_t st;  // the stream the scope's work was queued on
};
static bool g_kt_on = false;
bool ktime_on() { return g_kt_on; }
static std::vector<KtRec> g_kt;
static std::vector<cudaEvent_t> g_kt_pool;

static cudaEvent_t kt_event() {
  if (!g_kt_pool.empty()) {
    cudaEvent_t e = g_kt_pool.back();
    g_kt_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

KtScope::KtScope(const char *name, double flops, double bytes) : idx(-1) {
  if (!g_kt_on) return;
  KtRec r{name, kt_event(), kt_event(), flops, bytes, g_ctx.stream};
  cudaEventRecord(r.a, g_ctx.stream);
  g_kt.push_back(r);
  idx = (int)g_kt.size() - 1;
}

KtScope::~KtScope() {
  if (idx >= 0 && idx < (int)g_kt.size()) cudaEventRecord(g_kt[idx].b, g_ctx.stream);
}

template <typename T>
__global__ void fma_peak_kernel(T *out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int j = 0; j < 8; j++) x[j] = (T)(threadIdx.x + j);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = fma(x[j], a, b);
  }
  T s = 0;
#pragma unroll
  for (int j = 0; j < 8; j++) s += x[j];
  if (s == (T)-12345.678) out[threadIdx.x] = s;  // keeps the chain live
}

}  // namespace mgb

extern "C" {

int matgb_ktime_enable(int on) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  cudaStreamSynchronize(g_ctx.stream);
  for (auto &r : g_kt) {
    g_kt_pool.push_back(r.a);
    g_kt_pool.push_back(r.b);
  }
  g_kt.clear();
  g_kt_on = on != 0;
  return 0;
}

int matgb_ktime_get(int i, char *name, int cap, long long *launches,
                    double *ms, double *flops, double *bytes) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  MGB_CUDA(cudaStreamSynchronize(g_ctx.stream));
  std::vector<std::string> names;
  for (auto &r : g_kt) {
    bool seen = false;
    for (auto &n : names) seen |= (n == r.name);
    if (!seen) names.push_back(r.name);
  }
  if (i < 0 || i >= (int)names.size()) return 1;
  long long cnt = 0;
  double t = 0, f = 0, by = 0;
  for (auto &r : g_kt) {
    if (r.name != names[i]) continue;
    float e = 0;
    cudaEventElapsedTime(&e, r.a, r.b);
    cnt++;
    t += e;
    f += r.flops;
    by += r.bytes;
  }
  if (name && cap > 0) {
    strncpy(name, names[i].c_str(), cap - 1);
    name[cap - 1] = 0;
  }
  if (launches) *launches = cnt;
  if (ms) *ms = t;
  if (flops) *flops = f;
  if (bytes) *bytes = by;
  return 0;
}

int matgb_ktime_trace(int i, char *name, int cap, double *t0_ms, double *t1_ms,
                      int *stream) {
  if (!ctx()) return MATGB_ERR_NO_DEVICE;
  MGB_CUDA(cudaDeviceSynchronize());
  if (i < 0 || i >= (int)g_kt.size()) return 1;
  const KtRec &r = g_kt[i];
  float a = 0, b = 0;
  MGB_CUDA(cudaEventElapsedTime(&a, g_kt[0].a, r.a));
  MGB_CUDA(cudaEventElapsedTime(&b, g_kt[0].a, r.b));
  // streams numbered by first appearance in the record list
  int sid = 0;
  std::vector<cudaStream_t> seen;
  for (auto &q : g_kt) {
    bool dup = false;
    for (auto s : seen) dup |= s == q.st;
    if (!dup) seen.push_back(q.st);
    if (q.st == r.st) break;
  }
  for (size_t k = 0; k < seen.size(); k++)
    if (seen[k] == r.st) sid = (int)k;
  if (name && cap > 0) {
    strncpy(name, r.name.c_str(), cap - 1);
    name[cap - 1] = 0;
  }
  if (t0_ms) *t0_ms = a;
  if (t1_ms) *t1_ms = b;
  if (stream) *stream = sid;
  return 0;
}

double matgb_measure_fma_peak(int which) {
  Ctx *c = ctx();
  if (!c) return -1.0;
  void *out = nullptr;
  if (cudaMalloc(&out, 4096 * sizeof(double)) != cudaSuccess) return -1.0;
  const int blocks = c->sms * 8, threads = 256, iters = 1 << 14;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(a, c->stream);
    if (which == 0)
      fma_peak_kernel<float><<<blocks, threads, 0, c->stream>>>(
          (float *)out, iters, 0.999f, 0.001f);
    else
      fma_peak_kernel<double><<<blocks, threads, 0, c->stream>>>(
          (double *)out, iters / 8, 0.999, 0.001);
    cudaEventRecord(b, c->stream);
    cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    if (ms < best) best = ms;
  }
  launched("fma_peak");
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  double it = which == 0 ? iters : iters / 8;
  double flops = 2.0 * 8 * it * (double)blocks * threads;
  return flops / (best * 1e-3) / 1e12;
}

}  // extern "C"
