// common.cu -- error state, launch counter, device scan and buffer helper.
#include <stdarg.h>
#include <stdio.h>
#include <atomic>
#include <mutex>
#include <vector>

#include "gcsph_common.cuh"

namespace gcsph {

static thread_local std::string g_last_error;
static std::atomic<unsigned long long> g_launches{0};

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  set_error("CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e), what, file, line);
  return e == cudaErrorMemoryAllocation ? GCSPH_ENOMEM : GCSPH_ECUDA;
}

void count_launch(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

// ---------------------------------------------------------------------------
// timers
// ---------------------------------------------------------------------------
static const char* kTimerNames[T_COUNT] = {"stage1", "stage2", "dpc", "xsph", "cspm",  "sort",
                                            "pairs",  "state",  "post", "dt",   "rowsum"};
struct TimerState {
  std::mutex mu;
  bool on = false;
  long long launches[T_COUNT] = {0};
  double ms[T_COUNT] = {0};
  struct Pending { int id; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t open[T_COUNT] = {nullptr};
  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
};
static TimerState g_timer;

bool timing_on() { return g_timer.on; }

static thread_local std::vector<TimerRec>* t_sink = nullptr;
static thread_local cudaEvent_t t_open[T_COUNT];

void timer_capture_to(std::vector<TimerRec>* sink) {
  t_sink = sink;
  for (int i = 0; i < T_COUNT; ++i) t_open[i] = nullptr;
}

void timer_account(const std::vector<TimerRec>& recs) {
  if (!g_timer.on || recs.empty()) return;
  std::lock_guard<std::mutex> lk(g_timer.mu);
  for (const TimerRec& r : recs) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess) continue;
    g_timer.ms[r.id] += ms;
    g_timer.launches[r.id] += 1;
  }
  cudaGetLastError();
}

void timer_release(std::vector<TimerRec>& recs) {
  for (TimerRec& r : recs) {
    if (r.a) cudaEventDestroy(r.a);
    if (r.b) cudaEventDestroy(r.b);
  }
  recs.clear();
}

void timer_begin(int id, cudaStream_t s) {
  if (!g_timer.on) return;
  if (t_sink) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return;
    cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    t_open[id] = e;
    return;
  }
  std::lock_guard<std::mutex> lk(g_timer.mu);
  cudaEvent_t e = g_timer.get();
  cudaEventRecord(e, s);
  g_timer.open[id] = e;
}

void timer_end(int id, cudaStream_t s) {
  if (!g_timer.on) return;
  if (t_sink) {
    cudaEvent_t a = t_open[id];
    if (!a) return;
    cudaEvent_t b = nullptr;
    if (cudaEventCreate(&b) != cudaSuccess) return;
    cudaEventRecordWithFlags(b, s, cudaEventRecordExternal);
    t_sink->push_back({id, a, b});
    t_open[id] = nullptr;
    return;
  }
  std::lock_guard<std::mutex> lk(g_timer.mu);
  cudaEvent_t a = g_timer.open[id];
  if (!a) return;
  cudaEvent_t b = g_timer.get();
  cudaEventRecord(b, s);
  g_timer.pending.push_back({id, a, b});
  g_timer.open[id] = nullptr;
}

void timer_collect() {
  if (!g_timer.on) return;
  std::lock_guard<std::mutex> lk(g_timer.mu);
  std::vector<TimerState::Pending> keep;
  for (auto& p : g_timer.pending) {
    if (cudaEventQuery(p.b) != cudaSuccess) { keep.push_back(p); continue; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    g_timer.ms[p.id] += ms;
    g_timer.launches[p.id] += 1;
    g_timer.pool.push_back(p.a);
    g_timer.pool.push_back(p.b);
  }
  cudaGetLastError();
  g_timer.pending.swap(keep);
}

int DevBuf::ensure(size_t need, cudaStream_t s, bool zero) {
  if (need == 0) need = 16;
  if (bytes < need) {
    if (p) {
      cudaError_t e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize", __FILE__, __LINE__);
      cudaFree(p);
      p = nullptr;
      bytes = 0;
    }
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
      p = nullptr;
      return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
    }
    bytes = need;
  }
  if (zero) {
    cudaError_t e = cudaMemsetAsync(p, 0, need, s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync", __FILE__, __LINE__);
  }
  return GCSPH_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

// ---------------------------------------------------------------------------
// Exclusive scan: 256 threads x 8 items per block, block totals scanned
// recursively, then added back.  No block ever waits on another block.
// ---------------------------------------------------------------------------

template <class TIn, class TOut>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile(const TIn* __restrict__ in, TOut* __restrict__ out,
                                                            int64_t n_in, int64_t m, int64_t* __restrict__ bsum) {
  __shared__ long long wtot[SCAN_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)tid * SCAN_ITEMS;
  long long v[SCAN_ITEMS];
  long long s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int64_t idx = base + j;
    long long x = idx < n_in ? (long long)in[idx] : 0;
    v[j] = s;
    s += x;
  }
  long long inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) wtot[w] = inc;
  __syncthreads();
  if (w == 0) {
    long long t = lane < SCAN_THREADS / 32 ? wtot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < SCAN_THREADS / 32) wtot[lane] = t;
  }
  __syncthreads();
  long long woff = w > 0 ? wtot[w - 1] : 0;
  long long excl = woff + inc - s;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    int64_t idx = base + j;
    if (idx < m) out[idx] = (TOut)(excl + v[j]);
  }
  if (tid == 0) bsum[blockIdx.x] = wtot[SCAN_THREADS / 32 - 1];
}

template <class TOut>
__global__ void k_scan_add(TOut* __restrict__ out, int64_t m, const int64_t* __restrict__ boff) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = (TOut)((long long)out[i] + boff[i / SCAN_TILE]);
}

// one block walks the whole array in tiles of 1024 x 8 items, carrying the
// running total: a single launch for the small arrays of small problems.
// Each tile is loaded coalesced into shared memory, then every thread scans
// its 8 consecutive items.  Block b scans array b of up to two (in0/out0,
// in1/out1), so two scans of one size share a launch.
template <class TIn, class TOut>
__global__ void __launch_bounds__(1024) k_scan_single(const TIn* __restrict__ in0, TOut* __restrict__ out0,
                                                      const TIn* __restrict__ in1, TOut* __restrict__ out1,
                                                      int64_t n_in, int64_t m) {
  constexpr int TILE = 1024 * SCAN_ITEMS;
  // 32-bit inputs go through shared memory (32 KB); 64-bit ones (block totals) are read directly
  constexpr bool SMEM = sizeof(TIn) == 4;
  __shared__ int tile[SMEM ? TILE : 1];
  __shared__ long long wtot[32];
  const TIn* __restrict__ in = blockIdx.x == 0 ? in0 : in1;
  TOut* __restrict__ out = blockIdx.x == 0 ? out0 : out1;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  long long carry = 0;
  for (int64_t tile0 = 0; tile0 < m; tile0 += TILE) {
    if constexpr (SMEM) {
#pragma unroll
      for (int j = 0; j < SCAN_ITEMS; ++j) {
        const int64_t idx = tile0 + (int64_t)j * 1024 + tid;
        tile[j * 1024 + tid] = idx < n_in ? (int)in[idx] : 0;
      }
      __syncthreads();
    }
    long long v[SCAN_ITEMS];
    long long s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
      long long x;
      if constexpr (SMEM) {
        x = (long long)tile[tid * SCAN_ITEMS + j];
      } else {
        const int64_t idx = tile0 + (int64_t)tid * SCAN_ITEMS + j;
        x = idx < n_in ? (long long)in[idx] : 0;
      }
      v[j] = s;
      s += x;
    }
    long long inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) wtot[w] = inc;
    __syncthreads();
    if (w == 0) {
      long long t = wtot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      wtot[lane] = t;
    }
    __syncthreads();
    const long long excl = carry + (w > 0 ? wtot[w - 1] : 0) + inc - s;
    const int64_t base = tile0 + (int64_t)tid * SCAN_ITEMS;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
      const int64_t idx = base + j;
      if (idx < m) out[idx] = (TOut)(excl + v[j]);
    }
    carry += wtot[31];
    __syncthreads();
  }
}

template <class TIn, class TOut>
static int scan_impl(const TIn* in, TOut* out, int64_t n_in, int64_t m, int64_t* scratch, cudaStream_t s) {
  if (m <= SCAN_SINGLE_MAX) {
    k_scan_single<TIn, TOut><<<1, 1024, 0, s>>>(in, out, nullptr, nullptr, n_in, m);
    GC_LAUNCHED();
    return GCSPH_OK;
  }
  int64_t nb = (m + SCAN_TILE - 1) / SCAN_TILE;
  if (nb < 1) nb = 1;
  if (nb > 0x7fffffffLL) return fail(GCSPH_EINVAL, "scan too large");
  k_scan_tile<TIn, TOut><<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n_in, m, scratch);
  GC_LAUNCHED();
  if (nb == 1) return GCSPH_OK;
  int64_t* bscan = scratch + nb;
  int rc = scan_impl<int64_t, int64_t>(scratch, bscan, nb, nb, bscan + nb + 1, s);
  if (rc) return rc;
  k_scan_add<TOut><<<nblocks(m, 256), 256, 0, s>>>(out, m, bscan);
  GC_LAUNCHED();
  return GCSPH_OK;
}

int exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, int64_t* scratch, cudaStream_t s) {
  return scan_impl<int32_t, int64_t>(in, out, n, n + 1, scratch, s);
}
int exclusive_scan_i32_to_i32(const int32_t* in, int32_t* out, int64_t n, int64_t* scratch, cudaStream_t s) {
  return scan_impl<int32_t, int32_t>(in, out, n, n + 1, scratch, s);
}
int exclusive_scan2_i32_to_i64(const int32_t* in0, int64_t* out0, const int32_t* in1, int64_t* out1, int64_t n,
                               int64_t* scratch, cudaStream_t s) {
  if (n + 1 <= SCAN_SINGLE_MAX) {
    k_scan_single<int32_t, int64_t><<<2, 1024, 0, s>>>(in0, out0, in1, out1, n, n + 1);
    GC_LAUNCHED();
    return GCSPH_OK;
  }
  int rc = scan_impl<int32_t, int64_t>(in0, out0, n, n + 1, scratch, s);
  if (rc) return rc;
  return scan_impl<int32_t, int64_t>(in1, out1, n, n + 1, scratch, s);
}

int scan_preload() {
  cudaFuncAttributes a;
  const void* fns[] = {
      (const void*)k_scan_single<int32_t, int32_t>, (const void*)k_scan_single<int32_t, int64_t>,
      (const void*)k_scan_single<int64_t, int64_t>, (const void*)k_scan_tile<int32_t, int32_t>,
      (const void*)k_scan_tile<int32_t, int64_t>,   (const void*)k_scan_tile<int64_t, int64_t>,
      (const void*)k_scan_add<int32_t>,             (const void*)k_scan_add<int64_t>};
  for (const void* f : fns) GC_CUDA(cudaFuncGetAttributes(&a, f));
  return GCSPH_OK;
}

}  // namespace gcsph

extern "C" {
const char* gcsph_last_error(void) { return gcsph::g_last_error.c_str(); }
int gcsph_version(void) { return 1; }
uint64_t gcsph_launch_count(void) { return gcsph::g_launches.load(); }

int gcsph_timing_enable(int on) {
  gcsph::g_timer.on = on != 0;
  return GCSPH_OK;
}
int gcsph_timing_reset(void) {
  gcsph::timer_collect();
  std::lock_guard<std::mutex> lk(gcsph::g_timer.mu);
  for (int i = 0; i < gcsph::T_COUNT; ++i) { gcsph::g_timer.launches[i] = 0; gcsph::g_timer.ms[i] = 0; }
  return GCSPH_OK;
}
int gcsph_timing_count(void) { return gcsph::T_COUNT; }
const char* gcsph_timing_name(int32_t id) {
  return (id >= 0 && id < gcsph::T_COUNT) ? gcsph::kTimerNames[id] : "";
}
int gcsph_timing_get(int32_t id, int64_t* launches, double* total_ms) {
  if (id < 0 || id >= gcsph::T_COUNT) return gcsph::fail(GCSPH_EINVAL, "bad timer id %d", (int)id);
  gcsph::timer_collect();
  std::lock_guard<std::mutex> lk(gcsph::g_timer.mu);
  if (launches) *launches = gcsph::g_timer.launches[id];
  if (total_ms) *total_ms = gcsph::g_timer.ms[id];
  return GCSPH_OK;
}
}
