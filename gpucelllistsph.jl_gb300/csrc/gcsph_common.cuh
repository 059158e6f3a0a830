// gcsph_common.cuh -- shared device math and host plumbing for libgcsph.so.
//
// The FP64 drop-in path is compiled with -fmad=false so that every expression
// below rounds exactly like the reference's Julia source (left-to-right, no
// contraction); the CPU oracle uses the same operation order, so the two agree
// bit-for-bit up to summation order and libm's cos.
#pragma once
#include <vector>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <string>

#include "../../include/gcsph.h"

// Float64(pi), the value Julia uses for the Irrational pi.
#define GCSPH_PI64 3.141592653589793

namespace gcsph {

// ----------------------------------------------------------------------------
// error reporting (thread-local last error, int status codes at the ABI)
// ----------------------------------------------------------------------------
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);
void count_launch(int n = 1);

#define GC_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess) return ::gcsph::cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)

#define GC_LAUNCHED()                                                          \
  do {                                                                         \
    ::gcsph::count_launch();                                                   \
    cudaError_t _e = cudaPeekAtLastError();                                    \
    if (_e != cudaSuccess) return ::gcsph::cuda_fail(_e, "kernel launch", __FILE__, __LINE__); \
  } while (0)

inline int nblocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (int)(b < 1 ? 1 : b);
}

// ----------------------------------------------------------------------------
// WendlandC2 (SPHKernels.jl 2.2, published formula; call sites
// src/gpukernels_sph.jl:95,150,207,343,1490,1519).  u = r * Hinv.
//   W  = sigma_D Hinv^D     (1-u)^4 (1+4u)   for u < 1
//   dW = sigma_D Hinv^(D+1) (-20 u (1-u)^3)  for u < 1
// sigma_2 = 7/pi, sigma_3 = 21/(2 pi).
// ----------------------------------------------------------------------------
template <int D>
__host__ __device__ inline double wc2_sigma() {
  return D == 2 ? 7.0 / GCSPH_PI64 : 21.0 / (2.0 * GCSPH_PI64);
}
template <int D>
__host__ __device__ inline double wc2_norm_w(double Hinv) {
  double p = Hinv;
  for (int k = 1; k < D; ++k) p = p * Hinv;
  return wc2_sigma<D>() * p;
}
template <int D>
__host__ __device__ inline double wc2_norm_dw(double Hinv) {
  double p = Hinv;
  for (int k = 1; k < D + 1; ++k) p = p * Hinv;
  return wc2_sigma<D>() * p;
}
// nW = wc2_norm_w<D>(Hinv) precomputed once per launch
__host__ __device__ inline double wc2_w(double u, double nW) {
  if (!(u < 1.0)) return 0.0;
  double t = 1.0 - u;
  double t2 = t * t;
  double t4 = t2 * t2;
  return ((1.0 + 4.0 * u) * t4) * nW;
}
__host__ __device__ inline double wc2_dw(double u, double nDW) {
  if (!(u < 1.0)) return 0.0;
  double t = 1.0 - u;
  double t3 = (t * t) * t;
  return ((-20.0 * u) * t3) * nDW;
}

// powfancy7th, src/gpukernels_sph.jl:499-515 (bit-trick guess + 2 Newton steps)
__host__ __device__ inline double powfancy7th(double x, double ginv, int gamma) {
  if (gamma == 7) {
    double ax = fabs(x);
#ifdef __CUDA_ARCH__
    unsigned long long bits = (unsigned long long)__double_as_longlong(ax);
    bits = 0x36cd000000000000ULL + bits / 7ULL;
    double t = __longlong_as_double((long long)bits);
#else
    uint64_t bits;
    memcpy(&bits, &ax, 8);
    bits = 0x36cd000000000000ULL + bits / 7ULL;
    double t;
    memcpy(&t, &bits, 8);
#endif
    t = copysign(t, x);
    for (int it = 0; it < 2; ++it) {
      double t2 = t * t;
      double t3 = t2 * t;
      double t4 = t2 * t2;
      double xot4 = x / t4;
      t = t - (t * (t3 - xot4)) / (4.0 * t3 + 3.0 * xot4);
    }
    return t;
  }
  return pow(x, ginv);
}

#define GC_INLINE __host__ __device__ inline
/* cos(x) by Cody-Waite reduction modulo pi/2 (pi/2 split into a 33-bit head
 * and its tail) and the Taylor series of cos / sin on |r| <= pi/4 (terms to
 * r^16 / r^17) in Horner form in r^2.  Plain IEEE operations without FMA, so
 * the CPU oracle and the CUDA kernels produce the same bits; |x| < 2^20 pi/2
 * keeps k*head exact.  Used for the surface-tension cosine (∂v∂tpF!). */
GC_INLINE double gc_cos(double x) {
  const double PIO2_HI = 1.5707963267341256;    /* 0x3FF921FB54400000 */
  const double PIO2_LO = 6.077100506506192e-11; /* pi/2 - PIO2_HI */
  const double INV_PIO2 = 0.6366197723675814;
  double kd = floor(x * INV_PIO2 + 0.5);
  double r = (x - kd * PIO2_HI) - kd * PIO2_LO;
  double z = r * r;
  double c = 1.0 + z * (-0.5 + z * (0.041666666666666664 + z * (-0.001388888888888889 +
             z * (2.48015873015873e-05 + z * (-2.755731922398589e-07 + z * (2.08767569878681e-09 +
             z * (-1.1470745597729725e-11 + z * 4.779477332387385e-14)))))));
  double s = r + r * z * (-0.16666666666666666 + z * (0.008333333333333333 + z * (-0.0001984126984126984 +
             z * (2.7557319223985893e-06 + z * (-2.505210838544172e-08 + z * (1.6059043836821613e-10 +
             z * (-7.647163731819816e-13 + z * 2.8114572543455206e-15)))))));
  long long k = (long long)kd;
  switch ((int)(k & 3)) {
    case 0: return c;
    case 1: return -s;
    case 2: return -c;
    default: return s;
  }
}

// Float64 ^ Int of the Tait EOS: gamma == 7 as ((x2*x2)*x2)*x, otherwise
// left-to-right products (same sequence as the oracle).
__host__ __device__ inline double ipow(double x, int n) {
  if (n == 7) {
    double x2 = x * x, x4 = x2 * x2, x6 = x4 * x2;
    return x6 * x;
  }
  if (n == 0) return 1.0;
  double r = x;
  int m = n < 0 ? -n : n;
  for (int k = 1; k < m; ++k) r = r * x;
  return n < 0 ? 1.0 / r : r;
}

// pressure(), src/gpukernels_sph.jl:691-697
__host__ __device__ inline double eos(double rho, int gamma, double rho0, double P0, int pt) {
  if (pt <= 1 && rho < rho0) return 0.0;
  return P0 * (ipow(rho / rho0, gamma) - 1.0);
}

// positive doubles order like their bit patterns: atomicMax on the bits
__device__ inline void atomic_max_pos(unsigned long long* addr, double v) {
  if (!(v > 0.0)) return;
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

// Warp/block max of a non-negative double, one atomic per block
__device__ inline double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ----------------------------------------------------------------------------
// device exclusive scan (3 phases, no inter-block waiting)
// ----------------------------------------------------------------------------
// out[i] = sum_{j<i} in[j] for i in [0, n]; out[n] = total.  scratch must
// hold scan_scratch_elems(n + 1) int64 values.  Arrays of up to
// SCAN_SINGLE_MAX items take one single-block launch; longer ones are
// scanned in tiles of SCAN_TILE items, with the tile totals scanned
// recursively in the scratch.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int64_t SCAN_TILE = (int64_t)SCAN_THREADS * SCAN_ITEMS;
constexpr int64_t SCAN_SINGLE_MAX = 65536;
constexpr int64_t scan_scratch_elems(int64_t m) {
  return (m + SCAN_TILE - 1) / SCAN_TILE <= 1
             ? 1
             : 2 * ((m + SCAN_TILE - 1) / SCAN_TILE) + 1 + scan_scratch_elems((m + SCAN_TILE - 1) / SCAN_TILE);
}
// load every scan kernel into the current context now (a process with lazy
// module loading otherwise loads each at its first launch, which needs
// device memory for its code)
int scan_preload();

// Arrays of up to SCAN_FOLD_MAX items are scanned by the last block of the
// kernel that produced them (block_exclusive_scan), which saves the scan's
// own launch: a step at small N is bound by its chain of short launches.
constexpr int64_t SCAN_FOLD_MAX = 16384;

// true in every thread of the block that finishes last among gridDim.x
// blocks; each thread's earlier global writes are visible to that block.
// *cnt counts finished blocks and is reset to 0 by the last one.  The block
// barrier orders its threads' writes before thread 0's device-scope fence,
// whose release is cumulative, so one fence per block suffices (the pattern
// of a cooperative grid barrier).
__device__ inline bool last_block_of_grid(unsigned* cnt) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(cnt, 1u) == gridDim.x - 1;
    if (s_last) {
      __threadfence();
      *cnt = 0u;
    }
  }
  __syncthreads();
  return s_last != 0;
}

// out[i] = sum_{j<i} in[j] for i in [0, n] (out[n] = total), by one block
// (blockDim.x a multiple of 32), 16 items per thread per tile, read as four
// 16-byte vectors (in 16-byte aligned).  Reads go to L2 (ld.global.cg): the
// inputs were written by other blocks of the grid.
template <class TOut>
__device__ void block_exclusive_scan(const int32_t* in, TOut* out, int64_t n) {
  constexpr int IT = 16;
  __shared__ long long wsum[32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  long long carry = 0;
  for (int64_t base = 0; base <= n; base += (int64_t)blockDim.x * IT) {
    const int64_t i0 = base + (int64_t)tid * IT;
    int v[IT];
    if (i0 + IT <= n) {
#pragma unroll
      for (int q = 0; q < IT / 4; ++q) {
        const int4 t = __ldcg(reinterpret_cast<const int4*>(in + i0) + q);
        v[4 * q] = t.x;
        v[4 * q + 1] = t.y;
        v[4 * q + 2] = t.z;
        v[4 * q + 3] = t.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < IT; ++j) v[j] = i0 + j < n ? __ldcg(in + i0 + j) : 0;
    }
    long long s = 0;
#pragma unroll
    for (int j = 0; j < IT; ++j) s += v[j];
    long long inc = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
      long long t = lane < nw ? wsum[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      if (lane < nw) wsum[lane] = t;
    }
    __syncthreads();
    long long run = carry + (w > 0 ? wsum[w - 1] : 0) + inc - s;
#pragma unroll
    for (int j = 0; j < IT; ++j) {
      if (i0 + j <= n) out[i0 + j] = (TOut)run;
      run += v[j];
    }
    carry += wsum[nw - 1];
    __syncthreads();
  }
}

int exclusive_scan_i32_to_i64(const int32_t* in, int64_t* out, int64_t n, int64_t* scratch,
                              cudaStream_t s);
int exclusive_scan_i32_to_i32(const int32_t* in, int32_t* out, int64_t n, int64_t* scratch,
                              cudaStream_t s);
// two scans of n items each (one launch when they are small)
int exclusive_scan2_i32_to_i64(const int32_t* in0, int64_t* out0, const int32_t* in1, int64_t* out1, int64_t n,
                               int64_t* scratch, cudaStream_t s);

// ----------------------------------------------------------------------------
// per-kernel-family CUDA-event timers (off unless gcsph_timing_enable(1))
// ----------------------------------------------------------------------------
enum TimerId {
  T_STAGE1 = 0, T_STAGE2, T_DPC, T_XSPH, T_CSPM, T_SORT, T_PAIRS, T_STATE, T_POST, T_DT, T_ROWSUM, T_COUNT
};
bool timing_on();
void timer_begin(int id, cudaStream_t s);
void timer_end(int id, cudaStream_t s);
void timer_collect();  // after a stream sync: fold finished event pairs into the totals
// timers inside a captured graph: while a sink is set, timer_begin/timer_end
// record external event nodes into the capture and list them in the sink;
// after each replay has finished, timer_account folds their intervals in
struct TimerRec {
  int id;
  cudaEvent_t a, b;
};
void timer_capture_to(std::vector<TimerRec>* sink);
void timer_account(const std::vector<TimerRec>& recs);
void timer_release(std::vector<TimerRec>& recs);

// device buffer helper
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t need, cudaStream_t s, bool zero = false);
  void release();
  template <class T> T* as() const { return (T*)p; }
};

}  // namespace gcsph
