// celllist.cu -- GPUCellList on sm_103a: frozen grid, counting sort of the
// particles into cell order, and the pair set as a neighbour CSR.
//
// Reference behaviour restated (src/celllist.jl, src/gpukernels_cls.jl):
//  * grid frozen at construction: cs raised to dist, MIN lowered by
//    |(MIN+sqrt(eps))*sqrt(eps)|, CELL = ceil((MAX-MIN)/cs)   (celllist.jl:27-46)
//  * cell of a point: ceil(Int32, clamp((x-MIN)*(1/cs), 1, CELL))
//    (gpukernels_cls.jl:29-60); out-of-box points land in edge cells
//  * pair set: every (i,j), i != j, whose cells are within Chebyshev distance
//    1 and whose r^2 = (xi-xj)^2 + (yi-yj)^2 [+ (zi-zj)^2], evaluated left to
//    right without FMA, is < dist^2 (neib_internal! + the half-stencil
//    neib_external! launches, gpukernels_cls.jl:293-587)
// The reference scatters pairs with per-cell threads and global atomics; here
// each sorted particle scans the 3^D stencil as 3^(D-1) contiguous x-rows of
// the sorted arrays and the pairs land at scanned offsets, so the emitted list
// is deterministic (ascending sorted index).
#include <mutex>
#include <utility>

#include <stdint.h>
#include "celllist.cuh"

namespace gcsph {

static constexpr int TPB = 256;

// ---------------------------------------------------------------------------
// min/max reduction for the grid bounds (celllist.jl:41-43), every dimension
// in one launch (blockIdx.y = dimension).  Julia's minimum/maximum propagate
// NaN and the constructor's ceil(Int, NaN) then throws; a NaN coordinate
// makes that block's minimum NaN so that the host can refuse the set.
// ---------------------------------------------------------------------------
__global__ void k_minmax(const double* __restrict__ x0, const double* __restrict__ x1,
                         const double* __restrict__ x2, int64_t N, double* __restrict__ part) {
  const double* __restrict__ x = blockIdx.y == 0 ? x0 : (blockIdx.y == 1 ? x1 : x2);
  double mn = INFINITY, mx = -INFINITY;
  bool nan = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    double v = x[i];
    nan |= v != v;
    mn = fmin(mn, v);
    mx = fmax(mx, v);
  }
  nan = __any_sync(0xffffffffu, nan);
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  __shared__ double smn[TPB / 32], smx[TPB / 32];
  __shared__ int snan[TPB / 32];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { smn[w] = mn; smx[w] = mx; snan[w] = nan; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < TPB / 32; ++k) { mn = fmin(mn, smn[k]); mx = fmax(mx, smx[k]); nan |= snan[k] != 0; }
    double* p = part + 2 * ((int64_t)blockIdx.y * gridDim.x + blockIdx.x);
    p[0] = nan ? NAN : mn;
    p[1] = mx;
  }
}

// blocks of k_minmax per dimension: four per SM of the current device, at
// most MINMAX_MAX_BLOCKS
int minmax_blocks() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) {
    cudaGetLastError();
    sms = 1;
  }
  return 4 * sms < MINMAX_MAX_BLOCKS ? 4 * sms : MINMAX_MAX_BLOCKS;
}

// the bounding box of the D coordinate arrays: one launch, one read-back of
// the per-block partials (part_dev, part_host: 2 * D * nb doubles), one wait
int bounding_box(int D, const double* const* x, int64_t N, int nb, double* part_dev, double* part_host,
                 cudaStream_t st, double* mn, double* mx) {
  k_minmax<<<dim3(nb, D), TPB, 0, st>>>(x[0], x[1], D == 3 ? x[2] : x[0], N, part_dev);
  GC_LAUNCHED();
  GC_CUDA(cudaMemcpyAsync(part_host, part_dev, sizeof(double) * 2 * D * nb, cudaMemcpyDeviceToHost, st));
  GC_CUDA(cudaStreamSynchronize(st));
  for (int d = 0; d < D; ++d) {
    double a = INFINITY, b = -INFINITY;
    for (int k = 0; k < nb; ++k) {
      const double* p = part_host + 2 * ((int64_t)d * nb + k);
      if (p[0] != p[0]) return fail(GCSPH_EINVAL, "NaN coordinate in dimension %d: no cell grid", d + 1);
      a = fmin(a, p[0]);
      b = fmax(b, p[1]);
    }
    mn[d] = a;
    mx[d] = b;
  }
  return GCSPH_OK;
}

// ---------------------------------------------------------------------------
// binning: key, arrival slot, per-cell count (kernel_cellmap!)
// ---------------------------------------------------------------------------
// With fold_cnt the last block to finish also scans the counts into
// cellstart (grids of at most SCAN_FOLD_MAX - 1 cells): no separate scan.
// With popmax the largest population of a cell goes to *popmax (which the
// caller zeroed): one atomic per warp.
template <int D>
__global__ void k_cellkey(const double* __restrict__ x0, const double* __restrict__ x1, const double* __restrict__ x2,
                          int64_t N, Grid g, int32_t* __restrict__ key, int32_t* __restrict__ slot,
                          int32_t* __restrict__ count, int32_t* __restrict__ cellstart, unsigned* fold_cnt,
                          int* popmax) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int pop = 0;
  if (i < N) {
    const int32_t lin = cell_key<D>(x0, x1, x2, i, g);
    key[i] = lin;
    slot[i] = pop = atomicAdd(&count[lin], 1);
    ++pop;
  }
  if (popmax) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pop = max(pop, __shfl_xor_sync(0xffffffffu, pop, o));
    if ((threadIdx.x & 31) == 0 && pop > 0) atomicMax(popmax, pop);
  }
  if (fold_cnt && last_block_of_grid(fold_cnt)) {
    block_exclusive_scan<int32_t>(count, cellstart, g.ncell);
    // the counts are spent: zero again for the next binning (a cell's
    // population is cellstart[c + 1] - cellstart[c] from here on)
    __syncthreads();
    for (int64_t c = threadIdx.x; c < g.ncell; c += blockDim.x) count[c] = 0;
  }
}

// the arrival lists: point i at its cell's start plus its arrival slot; with
// tord also its order value (ord[i], or i), for rank_in_cell
__global__ void k_scatter_arrival(const int32_t* __restrict__ key, const int32_t* __restrict__ slot,
                                  const int32_t* __restrict__ cellstart, int64_t N, int32_t* __restrict__ tmp,
                                  const int32_t* __restrict__ ord = nullptr, int32_t* __restrict__ tord = nullptr) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int32_t pos = cellstart[key[i]] + slot[i];
  tmp[pos] = (int32_t)i;
  if (tord) tord[pos] = ord ? ord[i] : (int32_t)i;
}

// rank of each cell member by original index: stable, history-free order.
// Cost is sum over cells of n_c^2 integer compares (the reference's own pair
// search is quadratic per cell too).
__global__ void k_rank_in_cell(const int32_t* __restrict__ tmp, const int32_t* __restrict__ key,
                               const int32_t* __restrict__ cellstart, const int32_t* __restrict__ ord, int64_t N,
                               int32_t* __restrict__ perm) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= N) return;
  int32_t i = tmp[q];
  int32_t c = key[i];
  int32_t s = cellstart[c], e = cellstart[c + 1];
  int32_t oi = ord ? ord[i] : i;
  int32_t r = 0;
  for (int32_t t = s; t < e; ++t) {
    int32_t j = tmp[t];
    int32_t oj = ord ? ord[j] : j;
    r += (oj < oi);
  }
  perm[s + r] = i;
}

// the rank and its consequences in one pass: the point's slot in cell
// order, its key there and its original index (k_rank_in_cell then
// k_apply_perm, without the second launch)
__global__ void k_rank_apply(const int32_t* __restrict__ tmp, const int32_t* __restrict__ key,
                             const int32_t* __restrict__ cellstart, const int32_t* __restrict__ ord, int64_t N,
                             int32_t* __restrict__ perm, int32_t* __restrict__ skey, int32_t* __restrict__ orig,
                             const int32_t* __restrict__ tord) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= N) return;
  rank_in_cell(tmp, key, cellstart, ord, q, perm, skey, orig, nullptr, tord);
}

__global__ void k_apply_perm(const int32_t* __restrict__ perm, const int32_t* __restrict__ key,
                             const int32_t* __restrict__ ord, int64_t N, int32_t* __restrict__ skey,
                             int32_t* __restrict__ orig) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  int32_t i = perm[k];
  skey[k] = key[i];
  orig[k] = ord ? ord[i] : i;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of the cell keys (8-bit digits), the O(N) ordering of
// large sets.  Its input is the particles in original order (keys[o] is the
// key of the particle whose original index is o, vals[o] that particle), so
// sorting by key alone, stably, orders each cell by original index: the
// order the counting sort's in-cell rank gives, with no term in the square
// of a cell's population.  A tile is RADIX_TPB threads x RADIX_ITEMS keys.
// ---------------------------------------------------------------------------
constexpr int RADIX_TPB = 256;
constexpr int RADIX_ITEMS = 8;
constexpr int64_t RADIX_TILE = (int64_t)RADIX_TPB * RADIX_ITEMS;

// keys and values in original order: keys[ord[i]] = key[i], vals[ord[i]] = i
__global__ void k_radix_prep(const int32_t* __restrict__ key, const int32_t* __restrict__ ord, int64_t N,
                             int32_t* __restrict__ keys, int32_t* __restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int32_t o = ord[i];
  keys[o] = key[i];
  vals[o] = (int32_t)i;
}

// digit histogram of each tile, digit-major: hist[d * ntiles + tile]
__global__ void __launch_bounds__(RADIX_TPB) k_radix_up(const int32_t* __restrict__ keys, int64_t N, int shift,
                                                        int32_t* __restrict__ hist, int64_t ntiles) {
  __shared__ int h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * RADIX_TILE;
#pragma unroll
  for (int j = 0; j < RADIX_ITEMS; ++j) {
    const int64_t idx = base + (int64_t)j * RADIX_TPB + threadIdx.x;
    if (idx < N) atomicAdd(&h[(keys[idx] >> shift) & 255], 1);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// scatter of each tile's keys and values to their digit's scanned offset,
// stable: the tile's keys go in index order, RADIX_TPB at a time; lanes of a
// warp with equal digits rank by lane (match_any), warps by a prefix over
// the warps' counts, rounds by a running count per digit.  vals == nullptr:
// the value of key idx is idx.
__global__ void __launch_bounds__(RADIX_TPB) k_radix_down(const int32_t* __restrict__ keys,
                                                          const int32_t* __restrict__ vals, int64_t N, int shift,
                                                          const int32_t* __restrict__ offs, int64_t ntiles,
                                                          int32_t* __restrict__ keys_out,
                                                          int32_t* __restrict__ vals_out) {
  constexpr int NW = RADIX_TPB / 32;
  __shared__ int run[256];
  __shared__ int wcnt[NW][256];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  run[tid] = offs[(int64_t)tid * ntiles + blockIdx.x];
  const int64_t base = (int64_t)blockIdx.x * RADIX_TILE;
  const unsigned lt = (1u << lane) - 1u;
  for (int j = 0; j < RADIX_ITEMS; ++j) {
#pragma unroll
    for (int q = 0; q < NW; ++q) wcnt[q][tid] = 0;
    __syncthreads();
    const int64_t idx = base + (int64_t)j * RADIX_TPB + tid;
    const bool valid = idx < N;
    const int32_t kv = valid ? keys[idx] : 0;
    const int dg = valid ? ((kv >> shift) & 255) : 256;
    const unsigned peers = __match_any_sync(0xffffffffu, dg);
    const int rank = __popc(peers & lt);
    if (valid && rank == 0) wcnt[w][dg] = __popc(peers);
    __syncthreads();
    if (valid) {
      int pos = run[dg] + rank;
      for (int q = 0; q < w; ++q) pos += wcnt[q][dg];
      keys_out[pos] = kv;
      vals_out[pos] = vals ? vals[idx] : (int32_t)idx;
    }
    __syncthreads();
    int add = 0;
#pragma unroll
    for (int q = 0; q < NW; ++q) add += wcnt[q][tid];
    run[tid] += add;
  }
}

template <int D>
__global__ void k_gather_pos(const int32_t* __restrict__ idx, int64_t N, const double* __restrict__ a0,
                             const double* __restrict__ a1, const double* __restrict__ a2, double* __restrict__ b0,
                             double* __restrict__ b1, double* __restrict__ b2) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  int32_t i = idx[k];
  b0[k] = a0[i];
  b1[k] = a1[i];
  if (D == 3) b2[k] = a2[i];
}

// ---------------------------------------------------------------------------
// pair search over the 3^D stencil, as 3^(D-1) contiguous x-rows
// ---------------------------------------------------------------------------
template <int D>
__device__ inline double r2_ref(double ax, double ay, double az, double bx, double by, double bz) {
  double d0 = ax - bx;
  double d1 = ay - by;
  double s = d0 * d0 + d1 * d1;
  if (D == 3) {
    double d2 = az - bz;
    s = s + d2 * d2;
  }
  return s;
}

// MODE 0: count (full, up); MODE 1: fill nbr.  L lanes share one particle:
// the candidates of each x-row are tested L at a time, and the fill keeps the
// row ascending by compacting each round's hits with a sub-warp ballot.
template <int D, int MODE, int L>
__global__ void __launch_bounds__(TPB) k_pairs(const double* __restrict__ x0, const double* __restrict__ x1,
                                               const double* __restrict__ x2, const int32_t* __restrict__ skey,
                                               const int32_t* __restrict__ cellstart, int64_t N, Grid g,
                                               int32_t* __restrict__ cnt_full, int32_t* __restrict__ cnt_up,
                                               const int64_t* __restrict__ rs_full, int32_t* __restrict__ nbr) {
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;  // the whole sub-group leaves together
  const unsigned lanew = threadIdx.x & 31u;
  const unsigned gbase = lanew & ~(unsigned)(L - 1);
  const unsigned gm = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << gbase);
  const int nx = g.nc[0], ny = g.nc[1], nz = D == 3 ? g.nc[2] : 1;
  int32_t key = skey[k];
  int cx = key % nx;
  int t = key / nx;
  int cy = t % ny;
  int cz = t / ny;
  double ax = x0[k], ay = x1[k], az = D == 3 ? x2[k] : 0.0;
  int32_t nf = 0, nu = 0;
  int64_t wpos = MODE == 1 ? rs_full[k] : 0;
  const int xlo = cx > 0 ? cx - 1 : 0;
  const int xhi = cx < nx - 1 ? cx + 1 : nx - 1;
  for (int dz = (D == 3 ? -1 : 0); dz <= (D == 3 ? 1 : 0); ++dz) {
    int z = cz + dz;
    if (z < 0 || z >= nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = cy + dy;
      if (y < 0 || y >= ny) continue;
      int64_t base = (int64_t)nx * ((int64_t)y + (int64_t)ny * z);
      int32_t m0 = cellstart[base + xlo], m1 = cellstart[base + xhi + 1];
      for (int32_t mb = m0; mb < m1; mb += L) {
        const int32_t m = mb + lane;
        bool hit = false;
        if (m < m1 && m != k) {
          double r2 = r2_ref<D>(ax, ay, az, x0[m], x1[m], D == 3 ? x2[m] : 0.0);
          hit = r2 < g.dist2;
        }
        if (MODE == 0) {
          nf += hit;
          nu += hit && (m > k);
        } else {
          const unsigned bal = (__ballot_sync(gm, hit) >> gbase) & (L == 32 ? 0xffffffffu : ((1u << L) - 1u));
          if (hit) nbr[wpos + __popc(bal & ((1u << lane) - 1u))] = m;
          wpos += __popc(bal);
        }
      }
    }
  }
  if (MODE == 0) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
      nf += __shfl_xor_sync(gm, nf, o);
      nu += __shfl_xor_sync(gm, nu, o);
    }
    if (lane == 0) {
      cnt_full[k] = nf;
      cnt_up[k] = nu;
    }
  }
}

__global__ void k_emit_pairs(const int64_t* __restrict__ rs_full, const int64_t* __restrict__ rs_up,
                             const int32_t* __restrict__ nbr, const int32_t* __restrict__ orig, int64_t N, int64_t cap,
                             int32_t* __restrict__ pairs) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  int64_t r1 = rs_full[k + 1];
  int64_t u0 = rs_up[k], u1 = rs_up[k + 1];
  int64_t nu = u1 - u0;
  int32_t ok = orig[k] + 1;
  for (int64_t t = 0; t < nu; ++t) {
    int64_t pos = u0 + t;
    if (pos >= cap) break;
    int32_t om = orig[nbr[r1 - nu + t]] + 1;
    pairs[2 * pos] = ok < om ? ok : om;
    pairs[2 * pos + 1] = ok < om ? om : ok;
  }
}

// The same emit with L lanes per point: the row's entries are read
// contiguously and each pair is one 8-byte store (pairs 8-byte aligned), so a
// warp's loads and stores coalesce; same positions, same contents.
template <int L>
__global__ void k_emit_pairs_l(const int64_t* __restrict__ rs_full, const int64_t* __restrict__ rs_up,
                               const int32_t* __restrict__ nbr, const int32_t* __restrict__ orig, int64_t N,
                               int64_t cap, int2* __restrict__ pairs) {
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;
  const int64_t r1 = rs_full[k + 1];
  const int64_t u0 = rs_up[k], nu = rs_up[k + 1] - u0;
  const int32_t ok = orig[k] + 1;
  for (int64_t t = lane; t < nu; t += L) {
    const int64_t pos = u0 + t;
    if (pos >= cap) break;
    const int32_t om = orig[nbr[r1 - nu + t]] + 1;
    pairs[pos] = make_int2(ok < om ? ok : om, ok < om ? om : ok);
  }
}

// points per cell (cellpnum), from the cell starts
__global__ void k_cell_pop(const int32_t* __restrict__ cellstart, int64_t ncell, int32_t* __restrict__ pop) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncell) pop[c] = cellstart[c + 1] - cellstart[c];
}

// мaxpairs: n(n-1)/2 + n * (half-stencil neighbour counts), gpukernels_cls.jl:130-286
template <int D>
__global__ void k_maxpairs(const int32_t* __restrict__ cellstart, Grid g, unsigned long long* __restrict__ out) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long v = 0;
  auto count = [&](int64_t cell) -> int64_t { return cellstart[cell + 1] - cellstart[cell]; };
  if (c < g.ncell) {
    const int nx = g.nc[0], ny = g.nc[1], nz = D == 3 ? g.nc[2] : 1;
    int64_t n = count(c);
    if (n > 0) {
      int cx = (int)(c % nx);
      int64_t t = c / nx;
      int cy = (int)(t % ny), cz = (int)(t / ny);
      int64_t m = 0;
      const int no = D == 2 ? 4 : 13;
      const int off[13][3] = {{-1, 1, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {-1, 1, 1}, {0, 1, 1}, {1, 1, 1},
                              {1, 0, 1}, {0, 0, 1}, {-1, 1, -1}, {0, 1, -1}, {1, 1, -1}, {1, 0, -1}};
      for (int o = 0; o < no; ++o) {
        int a = cx + off[o][0], b = cy + off[o][1], z = cz + (D == 3 ? off[o][2] : 0);
        if (a >= 0 && a < nx && b >= 0 && b < ny && z >= 0 && z < nz)
          m += count(a + (int64_t)nx * (b + (int64_t)ny * z));
      }
      v = (unsigned long long)((int64_t)((double)(n * (n - 1)) * 0.5) + m * n);
    }
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int CellCore::read_scalar(const int64_t* dev, int64_t* host) {
  GC_CUDA(cudaMemcpyAsync(pin, dev, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GC_CUDA(cudaStreamSynchronize(st));
  *host = pin[0];
  return GCSPH_OK;
}

int CellCore::init(int D_, int64_t N_, const double* cellsize, double dist_, const double* MIN, const double* MAX,
                   const double* const* xin, cudaStream_t s) {
  D = D_;
  N = N_;
  dist = dist_;
  st = s;
  if (D != 2 && D != 3) return fail(GCSPH_EINVAL, "wrong dimention: D=%d (2 or 3)", D);
  if (N < 1 || N > 0x7ffffffeLL) return fail(GCSPH_EINVAL, "N=%lld out of range", (long long)N);
  if (!(dist > 0)) return fail(GCSPH_EINVAL, "dist must be > 0");
  GC_CUDA(cudaMallocHost((void**)&pin, 8 * sizeof(int64_t)));
  const double seps = 1.4901161193847656e-08;  // sqrt(eps(Float64)) = 2^-26
  double mn[3], mx[3];
  if (!MIN || !MAX) {
    const int nb = minmax_blocks();
    DevBuf part;
    int rc = part.ensure(sizeof(double) * 2 * D * nb, st);
    if (rc) return rc;
    double* hp = nullptr;
    GC_CUDA(cudaMallocHost((void**)&hp, sizeof(double) * 2 * D * nb));
    rc = bounding_box(D, xin, N, nb, part.as<double>(), hp, st, mn, mx);
    cudaFreeHost(hp);
    part.release();
    if (rc) return rc;
  }
  int64_t ncell = 1;
  for (int d = 0; d < D; ++d) {
    cs[d] = cellsize[d] < dist ? dist : cellsize[d];
    double lo = MIN ? MIN[d] : mn[d];
    double hi = MAX ? MAX[d] : mx[d];
    lo = lo - fabs((lo + seps) * seps);
    double c = ceil((hi - lo) / cs[d]);
    if (!(c >= 1.0) || c > 2.0e9) return fail(GCSPH_EINVAL, "degenerate grid in dim %d (CELL=%g)", d + 1, c);
    g.offset[d] = lo;
    g.hinv[d] = 1.0 / cs[d];
    g.nc[d] = (int)c;
    ncell *= (int64_t)c;
    if (ncell > 0x7ffffff0LL) return fail(GCSPH_EINVAL, "cell grid too large (%lld cells)", (long long)ncell);
  }
  for (int d = D; d < 3; ++d) { g.offset[d] = 0; g.hinv[d] = 0; g.nc[d] = 1; }
  g.D = D;
  g.ncell = ncell;
  g.dist2 = dist * dist;
  int rc;
  if ((rc = count.ensure(sizeof(int32_t) * ncell, st, true))) return rc;  // zero at rest
  if ((rc = cellstart.ensure(sizeof(int32_t) * (ncell + 1), st))) return rc;
  if ((rc = key.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = slot.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = tmp.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = tord.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = perm.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = skey.ensure(sizeof(int32_t) * N, st))) return rc;
  // the spare original-index map every binning writes into (then swapped in)
  if ((rc = orig_b.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = orig.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = cnt_full.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = cnt_up.ensure(sizeof(int32_t) * N, st))) return rc;
  if ((rc = rs_full.ensure(sizeof(int64_t) * (N + 1), st))) return rc;
  if ((rc = rs_up.ensure(sizeof(int64_t) * (N + 1), st))) return rc;
  int64_t sc = scan_scratch_elems((ncell > N ? ncell : N) + 1);
  if ((rc = scratch.ensure(sizeof(int64_t) * (sc + 16), st))) return rc;
  // zeroed once: each pass that folds a scan resets its counter itself
  if ((rc = foldcnt.ensure(sizeof(unsigned) * 2, st, true))) return rc;
  if (N + 1 <= SCAN_FOLD_MAX &&
      (rc = foldsum.ensure(sizeof(int32_t) * (2 * N + 4 * ROWS_FOLD_MAX_BLOCKS + 2), st)))
    return rc;
  if (N > RADIX_MIN_N) {
    const int64_t ntiles = (N + RADIX_TILE - 1) / RADIX_TILE;
    for (int b = 0; b < 2; ++b) {
      if ((rc = rkey[b].ensure(sizeof(int32_t) * N, st))) return rc;
      if ((rc = rval[b].ensure(sizeof(int32_t) * N, st))) return rc;
    }
    if ((rc = rhist.ensure(sizeof(int32_t) * 256 * ntiles, st))) return rc;
    if ((rc = rhoff.ensure(sizeof(int32_t) * (256 * ntiles + 1), st))) return rc;
    if ((rc = popmax.ensure(sizeof(int), st, true))) return rc;
    if (scan_scratch_elems(256 * ntiles + 1) > sc) return fail(GCSPH_EINVAL, "radix scan scratch");
  }
  return GCSPH_OK;
}

void CellCore::release() {
  DevBuf* all[] = {&count, &cellstart, &key, &slot, &tmp, &tord, &perm, &skey, &orig, &cnt_full, &cnt_up, &rs_full,
                   &rs_up, &nbr, &scratch, &pf[0], &pf[1], &pf[2], &pfmax, &pfthr, &pfcnt, &orig_b, &stage,
                   &foldcnt, &foldsum, &rkey[0], &rkey[1], &rval[0], &rval[1], &rhist, &rhoff, &popmax};
  for (DevBuf* b : all) b->release();
  if (pin) cudaFreeHost(pin);
  pin = nullptr;
}

int CellCore::sort(const double* const* xin, const int32_t* ord, bool may_sync, bool* rank_deferred,
                   bool keys_ready) {
  timer_begin(T_SORT, st);
  if (rank_deferred) *rank_deferred = false;
  if (keys_ready && !keys_in_step())
    return fail(GCSPH_ESTATE, "cell keys from the step for a set that does not take them");
  // count is zero at rest: every binning zeroes it again once scanned
  const double* x2 = D == 3 ? xin[2] : xin[0];
  int rc;
  const bool fold = g.ncell + 1 <= SCAN_FOLD_MAX;
  unsigned* fc = fold ? foldcnt.as<unsigned>() : nullptr;
  // large sets track the most crowded cell, which picks the in-cell ordering
  int* pm = N > RADIX_MIN_N ? popmax.as<int>() : nullptr;
  if (pm) GC_CUDA(cudaMemsetAsync(pm, 0, sizeof(int), st));
  // with keys_ready, key, slot and cellstart are written and count is zero again
  if (!keys_ready) {
    if (D == 2)
      k_cellkey<2><<<nblocks(N, TPB), TPB, 0, st>>>(xin[0], xin[1], x2, N, g, key.as<int32_t>(), slot.as<int32_t>(),
                                                     count.as<int32_t>(), cellstart.as<int32_t>(), fc, pm);
    else
      k_cellkey<3><<<nblocks(N, TPB), TPB, 0, st>>>(xin[0], xin[1], x2, N, g, key.as<int32_t>(), slot.as<int32_t>(),
                                                     count.as<int32_t>(), cellstart.as<int32_t>(), fc, pm);
    GC_LAUNCHED();
  }
  if (!fold) {
    rc = exclusive_scan_i32_to_i32(count.as<int32_t>(), cellstart.as<int32_t>(), g.ncell, scratch.as<int64_t>(), st);
    if (rc) return rc;
    GC_CUDA(cudaMemsetAsync(count.p, 0, sizeof(int32_t) * g.ncell, st));
  }
  if (pm && may_sync && sort_mode == 0 && (rc = read_popmax())) return rc;
  // the in-cell order: the counting sort's rank costs the square of a cell's
  // population per cell, the radix sort a fixed few passes over the set
  const bool radix = N > RADIX_MIN_N && (sort_mode == 2 || (sort_mode == 0 && last_popmax > RADIX_MIN_POP));
  // ord may be `orig` itself (re-sorting particles already in cell order), so
  // the new map is written to the spare buffer and the two are swapped
  int rc2 = orig_b.ensure(sizeof(int32_t) * N, st);
  if (rc2) return rc2;
  if (radix) {
    // crowded cells of a large set: the stable radix sort of the keys in original order
    const int64_t ntiles = (N + RADIX_TILE - 1) / RADIX_TILE;
    int bits = 1;
    while (bits < 31 && (1LL << bits) < g.ncell) ++bits;
    const int npass = (bits + 7) / 8;
    const int32_t* kin = key.as<int32_t>();
    const int32_t* vin = nullptr;
    int nxt = 0;
    if (ord) {
      k_radix_prep<<<nblocks(N, TPB), TPB, 0, st>>>(key.as<int32_t>(), ord, N, rkey[0].as<int32_t>(),
                                                     rval[0].as<int32_t>());
      GC_LAUNCHED();
      kin = rkey[0].as<int32_t>();
      vin = rval[0].as<int32_t>();
      nxt = 1;
    }
    for (int p = 0; p < npass; ++p) {
      k_radix_up<<<(unsigned)ntiles, RADIX_TPB, 0, st>>>(kin, N, 8 * p, rhist.as<int32_t>(), ntiles);
      GC_LAUNCHED();
      if ((rc = exclusive_scan_i32_to_i32(rhist.as<int32_t>(), rhoff.as<int32_t>(), 256 * ntiles,
                                          scratch.as<int64_t>(), st)))
        return rc;
      const bool last = p == npass - 1;
      int32_t* kout = last ? skey.as<int32_t>() : rkey[nxt].as<int32_t>();
      int32_t* vout = last ? perm.as<int32_t>() : rval[nxt].as<int32_t>();
      k_radix_down<<<(unsigned)ntiles, RADIX_TPB, 0, st>>>(kin, vin, N, 8 * p, rhoff.as<int32_t>(), ntiles, kout,
                                                            vout);
      GC_LAUNCHED();
      kin = kout;
      vin = vout;
      nxt ^= 1;
    }
    k_apply_perm<<<nblocks(N, TPB), TPB, 0, st>>>(perm.as<int32_t>(), key.as<int32_t>(), ord, N, skey.as<int32_t>(),
                                                   orig_b.as<int32_t>());
    GC_LAUNCHED();
  } else {
    // small sets: 64-thread blocks, so these latency-bound passes spread over more SMs
    const int tb = N <= RADIX_MIN_N ? 64 : TPB;
    k_scatter_arrival<<<nblocks(N, tb), tb, 0, st>>>(key.as<int32_t>(), slot.as<int32_t>(), cellstart.as<int32_t>(),
                                                      N, tmp.as<int32_t>(), ord, tord.as<int32_t>());
    GC_LAUNCHED();
    if (rank_deferred) {
      // the caller ranks (rank_in_cell) and applies the order in its own pass
      *rank_deferred = true;
      timer_end(T_SORT, st);
      return GCSPH_OK;
    }
    k_rank_apply<<<nblocks(N, tb), tb, 0, st>>>(tmp.as<int32_t>(), key.as<int32_t>(), cellstart.as<int32_t>(), ord, N,
                                                 perm.as<int32_t>(), skey.as<int32_t>(), orig_b.as<int32_t>(),
                                                 tord.as<int32_t>());
    GC_LAUNCHED();
  }
  sort_done();
  timer_end(T_SORT, st);
  return GCSPH_OK;
}

void CellCore::sort_done() {
  std::swap(orig.p, orig_b.p);
  std::swap(orig.bytes, orig_b.bytes);
  sorted = true;
  built = false;
  up_valid = false;
}

int CellCore::read_popmax() {
  if (N <= RADIX_MIN_N || !popmax.p) return GCSPH_OK;
  GC_CUDA(cudaMemcpyAsync(pin + 7, popmax.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GC_CUDA(cudaStreamSynchronize(st));
  const bool before = last_popmax > RADIX_MIN_POP;
  last_popmax = *(const int*)(pin + 7);
  // a captured step graph holds the ordering it was captured with: a change
  // of the choice retires the captured graphs
  if ((last_popmax > RADIX_MIN_POP) != before) ++gen;
  return GCSPH_OK;
}

int CellCore::gather_positions(const double* const* xin, double* const* xs) {
  const double* a2 = D == 3 ? xin[2] : xin[0];
  double* b2 = D == 3 ? xs[2] : xs[0];
  if (D == 2)
    k_gather_pos<2><<<nblocks(N, TPB), TPB, 0, st>>>(perm.as<int32_t>(), N, xin[0], xin[1], a2, xs[0], xs[1], b2);
  else
    k_gather_pos<3><<<nblocks(N, TPB), TPB, 0, st>>>(perm.as<int32_t>(), N, xin[0], xin[1], a2, xs[0], xs[1], b2);
  GC_LAUNCHED();
  return GCSPH_OK;
}

int CellCore::gather_positions_by_orig(const double* const* xorig, double* const* xs) {
  const double* a2 = D == 3 ? xorig[2] : xorig[0];
  double* b2 = D == 3 ? xs[2] : xs[0];
  if (D == 2)
    k_gather_pos<2><<<nblocks(N, TPB), TPB, 0, st>>>(orig.as<int32_t>(), N, xorig[0], xorig[1], a2, xs[0], xs[1], b2);
  else
    k_gather_pos<3><<<nblocks(N, TPB), TPB, 0, st>>>(orig.as<int32_t>(), N, xorig[0], xorig[1], a2, xs[0], xs[1], b2);
  GC_LAUNCHED();
  return GCSPH_OK;
}

// ---------------------------------------------------------------------------
// FP32 prefilter for the pair test.  GB300 issues 64x more FP32 than FP64
// instructions per cycle, so candidates are first tested on FP32 copies of
// (x - offset).  With B = max |x - offset| every FP32 coordinate is within
// 2^-24 B(1+2^-29) of its exact value, so with e0 = 2^-22 B (twice the
// worst case of a difference of two such coordinates plus its own rounding)
//   |r2f - r2| <= band = 2 e0 sqrt(D T') + D e0^2 + 2^-20 T'     (T' = 1.5 dist^2)
// covers the coordinate errors, the FP32 squares and sums and the FP64
// reference expression's own rounding for every candidate with r2 <= T'.
// A candidate is IN when r2f < T - band and OUT when r2f > T + band (both
// bounds rounded outwards); only candidates inside the band take the exact
// FP64 test of the reference, so the pair set is unchanged bit for bit.
// ---------------------------------------------------------------------------
template <int D>
__global__ void k_make_pf(const double* __restrict__ x0, const double* __restrict__ x1,
                          const double* __restrict__ x2, int64_t N, Grid g, float* __restrict__ f0,
                          float* __restrict__ f1, float* __restrict__ f2, unsigned long long* __restrict__ bmax,
                          float2* __restrict__ thr, unsigned* __restrict__ cnt) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double b = 0.0;
  if (k < N) {
    const double* X[3] = {x0, x1, x2};
    float* F[3] = {f0, f1, f2};
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double v = X[d][k] - g.offset[d];
      F[d][k] = (float)v;
      b = fmax(b, fabs(v));
    }
    if (b != b) b = INFINITY;  // NaN coordinate: every candidate of the set goes to FP64
  }
  b = warp_max(b);
  if ((threadIdx.x & 31) == 0) atomic_max_pos(bmax, b);
  pf_thresholds_last_block<D>(bmax, g.dist2, thr, cnt);
}


// Row starts of a small set as the count pass folds them (rows_fold, below)
struct FoldRows {
  // fb: local offsets [2N] (full, up), block totals [2G], block bases [2G],
  // the two totals [2]
  __device__ static int32_t* totals(int32_t* fb, int64_t N) { return fb + 2 * N; }
  __device__ static int32_t* bases(int32_t* fb, int64_t N, int G) { return fb + 2 * N + 2 * G; }
  // start of row i of array a (0 full, 1 up) as the fill pass reads it
  __device__ static int64_t start(const int32_t* fb, int a, int64_t i, int64_t N, int P, int G) {
    if (i >= N) return fb[2 * N + 4 * G + a];
    return (int64_t)fb[a * N + i] + fb[2 * N + 2 * G + a * G + i / P];
  }
};

// one point's row of the pair search with the FP32 prefilter (k_pairs32)
template <int D, int MODE, int L>
__device__ __forceinline__ void pairs32_row(const double* __restrict__ x0, const double* __restrict__ x1,
                                                 const double* __restrict__ x2, const float* __restrict__ f0,
                                                 const float* __restrict__ f1, const float* __restrict__ f2,
                                                 const float2* __restrict__ thr,
                                                 const int32_t* __restrict__ skey,
                                                 const int32_t* __restrict__ cellstart, int64_t N, Grid g,
                                                 int32_t* __restrict__ cnt_full, int32_t* __restrict__ cnt_up,
                                                 const int64_t* __restrict__ rs_full, int32_t* __restrict__ nbr,
                                                 int64_t cap, int* __restrict__ ovf, int32_t* __restrict__ stg,
                                                 int S, const int32_t* fold_buf, bool up) {
  // MODE 0: count; MODE 2: count and stage the row (ascending) in stg[k*S ..]
  // when it fits; MODE 1: fill the CSR row -- a copy of the staged row when
  // the count pass staged it, else the search again.  MODE 1 reads the row
  // starts from the count pass's fold buffer where it folded (FoldRows).
  // up: the half stencil, candidates m > k only (the cell list's own
  // (min, max) list): the rows whose cells all come before k's in key order
  // are skipped and k's own row starts at k + 1, so a row holds exactly the
  // larger-index part of the full row, in the same order
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;
  int64_t r0 = 0, r1 = 0;
  if (MODE == 1) {
    if (fold_buf) {
      r0 = FoldRows::start(fold_buf, 0, k, N, TPB / L, gridDim.x);
      r1 = FoldRows::start(fold_buf, 0, k + 1, N, TPB / L, gridDim.x);
    } else {
      r0 = rs_full[k];
      r1 = rs_full[k + 1];
    }
  }
  if (MODE == 1 && r1 > cap) {  // the row does not fit: report, write nothing
    if (ovf && lane == 0) atomicExch(ovf, 1);
    return;
  }
  if (MODE == 1 && stg) {
    const int32_t n = (int32_t)(r1 - r0);
    if (n <= S) {
      for (int32_t q = lane; q < n; q += L) nbr[r0 + q] = stg[k * S + q];
      return;
    }
  }
  const float2 tt = *thr;
  const float tlo = tt.x, thi = tt.y;
  const unsigned lanew = threadIdx.x & 31u;
  const unsigned gbase = lanew & ~(unsigned)(L - 1);
  const unsigned gm = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << gbase);
  const int nx = g.nc[0], ny = g.nc[1], nz = D == 3 ? g.nc[2] : 1;
  const int32_t key = skey[k];
  const int cx = key % nx;
  const int t = key / nx;
  const int cy = t % ny;
  const int cz = t / ny;
  const float ax = f0[k], ay = f1[k], az = D == 3 ? f2[k] : 0.0f;
  int32_t nf = 0, nu = 0;
  int64_t wpos = r0;
  int32_t spos = 0;  // MODE 2: staged entries so far
  const int xlo = cx > 0 ? cx - 1 : 0;
  const int xhi = cx < nx - 1 ? cx + 1 : nx - 1;
  // one candidate m per lane (valid: in range and not k itself); the ballot
  // keeps a group's hits in ascending m
  auto visit = [&](int32_t m, bool valid) {
    bool hit = false;
    if (valid) {
      const float d0 = ax - f0[m], d1 = ay - f1[m];
      float r2f = d0 * d0 + d1 * d1;
      if (D == 3) {
        const float d2 = az - f2[m];
        r2f = r2f + d2 * d2;
      }
      if (r2f < tlo) {
        hit = true;
      } else if (!(r2f > thi)) {  // inside the band (or NaN): the reference's FP64 test
        hit = r2_ref<D>(x0[k], x1[k], D == 3 ? x2[k] : 0.0, x0[m], x1[m], D == 3 ? x2[m] : 0.0) < g.dist2;
      }
    }
    if (MODE == 0) {
      nf += hit;
      nu += hit && (m > k);
    } else if (MODE == 2) {
      nf += hit;
      nu += hit && (m > k);
      const unsigned bal = (__ballot_sync(gm, hit) >> gbase) & (L == 32 ? 0xffffffffu : ((1u << L) - 1u));
      const int32_t at = spos + __popc(bal & ((1u << lane) - 1u));
      if (hit && at < S) stg[k * S + at] = m;
      spos += __popc(bal);
    } else {
      const unsigned bal = (__ballot_sync(gm, hit) >> gbase) & (L == 32 ? 0xffffffffu : ((1u << L) - 1u));
      if (hit) nbr[wpos + __popc(bal & ((1u << lane) - 1u))] = m;
      wpos += __popc(bal);
    }
  };
  if constexpr (D == 3) {
    // The point's nine rows of three cells, in key order, are one sequence of
    // candidates ascending in m: candidate t of it is m = t + dlt[r] for the
    // row r with cum[r] <= t < cum[r + 1].  The lanes stride the whole
    // sequence, so a group's trip count is ceil(candidates / L) rather than a
    // sum over rows of a few candidates each, and the groups of a warp do not
    // part at every row's end (measured on GB300: update! of 4M uniform 3-D
    // points 2.43 -> 2.27 ms; in 2-D, with tens of candidates per row, the
    // row-by-row walk below stays 4% faster)
    // The group's row table sits in shared memory; each lane keeps the row of
    // its candidate and moves on only where its candidate passes a row's end,
    // instead of locating every candidate among the nine rows (measured on
    // GB300: update! of 4M uniform 3-D points 2.28 -> 2.00 ms).
    constexpr int NR = 9;
    __shared__ int32_t s_rows[TPB / L][2 * NR + 1];  // starts (+ end sentinel), then m - t per row
    int32_t* rows = s_rows[threadIdx.x / L];
    int32_t tot = 0;
    if (lane == 0) {
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int z = cz + (r / 3 - 1), y = cy + (r % 3 - 1);
        int32_t m0 = 0, m1 = 0;
        if (z >= 0 && z < nz && y >= 0 && y < ny && !(up && r < NR / 2)) {
          const int64_t base = (int64_t)nx * ((int64_t)y + (int64_t)ny * z);
          m0 = cellstart[base + xlo];
          m1 = cellstart[base + xhi + 1];
          if (up && r == NR / 2) m0 = (int32_t)(k + 1);  // k's own row: k lies in it
        }
        rows[r] = tot;
        rows[NR + 1 + r] = m0 - tot;
        tot += m1 - m0;
      }
      rows[NR] = 0x7fffffff;
    }
    tot = __shfl_sync(gm, tot, gbase);
    __syncwarp(gm);
    int r = 0;
    int32_t next = rows[1], dd = rows[NR + 1];
    for (int32_t tb = 0; tb < tot; tb += L) {
      const int32_t t = tb + lane;
      while (t >= next) {  // r stops at the last row: its end is the sentinel
        ++r;
        next = rows[r + 1];
        dd = rows[NR + 1 + r];
      }
      const int32_t m = t + dd;
      visit(m, t < tot && m != k);
    }
  } else {
    // the three rows' candidate ranges first, so that their six loads go out
    // together rather than one row's after the previous row's candidates
    int32_t rm0[3], rm1[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int dy = r - 1, y = cy + dy;
      rm0[r] = rm1[r] = 0;
      if (!(up && dy < 0) && y >= 0 && y < ny) {
        const int64_t base = (int64_t)nx * (int64_t)y;
        rm0[r] = cellstart[base + xlo];
        rm1[r] = cellstart[base + xhi + 1];
        if (up && dy == 0) rm0[r] = (int32_t)(k + 1);  // k's own row: k lies in it
      }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int32_t m1 = rm1[r];
      for (int32_t mb = rm0[r]; mb < m1; mb += L) {
        const int32_t m = mb + lane;
        visit(m, m < m1 && m != k);
      }
    }
  }
  if (MODE != 1) {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) {
      nf += __shfl_xor_sync(gm, nf, o);
      nu += __shfl_xor_sync(gm, nu, o);
    }
    if (lane == 0) {
      cnt_full[k] = nf;
      cnt_up[k] = nu;
    }
  }
}

// MODE 3 (fill and pair list): the MODE 1 fill, then for each entry e of k's
// row whose neighbour m is above k the flat pair (k, m, e, mirror(e)), with
// mirror(e) the position of k in m's row, found by binary search in m's
// staged row (m's smaller-index part, ascending); a row too long to be staged
// gives mirror -1, which pass A resolves from the finished neighbour list.
template <int D, int L>
__device__ __forceinline__ void pairs32_quads(int64_t N, const int32_t* __restrict__ cnt_full,
                                              const int32_t* __restrict__ cnt_up, const int64_t* __restrict__ rs_full,
                                              const int64_t* __restrict__ rs_up, const int32_t* __restrict__ nbr,
                                              int64_t cap, const int32_t* __restrict__ stg, int S,
                                              int4* __restrict__ pq, const int32_t* fold_buf) {
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;
  // row starts as the fill read them (where the count pass folded them, the
  // final arrays are being written by this very pass)
  auto start = [&](int a, int64_t i) -> int64_t {
    return fold_buf ? FoldRows::start(fold_buf, a, i, N, TPB / L, gridDim.x) : (a ? rs_up : rs_full)[i];
  };
  // past the capacity the fill raised the overflow flag and the step is
  // repeated; the pair list holds cap / 2 + 1 pairs, enough when it fits
  if (start(0, N) > cap) return;
  const int64_t r0 = start(0, k), r1 = start(0, k + 1);
  const int32_t n = (int32_t)(r1 - r0);
  const int32_t nu = cnt_up[k];
  const int64_t u0 = start(1, k);
  const bool staged = n <= S;
  for (int32_t q = n - nu + lane; q < n; q += L) {
    const int32_t m = staged ? stg[k * S + q] : nbr[r0 + q];
    const int32_t nm = cnt_full[m];
    int32_t mir = -1;
    if (nm <= S) {
      int32_t lo = 0, hi = nm - cnt_up[m];
      const int32_t* row = stg + (int64_t)m * S;
      while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if (row[mid] < k) lo = mid + 1;
        else hi = mid;
      }
      mir = (int32_t)(start(0, m) + lo);
    }
    pq[u0 + (q - (n - nu))] = make_int4((int)k, (int)m, (int)(r0 + q), mir);
  }
}

// The row starts of small sets (N + 1 <= SCAN_FOLD_MAX), in two levels, in
// the int32 buffer fb (FoldRows below).  MODE 4's block b holds the points
// [b P, (b + 1) P), P = TPB / L: it scans their two counts into block-local
// offsets and stores its two totals; the last block to finish scans the G
// block totals into block bases.  The fill pass (MODE 1 / 3: same N and L,
// so the same G) reads a start as local offset + its block's base and writes
// the final rs_full / rs_up.  A single-block scan of all N counts walks them
// tile after tile, one load round trip each; this way the last block has one
// scan of G entries.  Sums fit in int32: N + 1 <= SCAN_FOLD_MAX points have
// fewer than 2^28 neighbour entries.

template <int L>
__device__ __forceinline__ void rows_fold(const int32_t* cnt_full, const int32_t* cnt_up, int64_t N,
                                          int64_t* rs_full, int64_t* rs_up, int32_t* fb, unsigned* fold_cnt) {
  constexpr int P = TPB / L, NW = TPB / 32, IT = ROWS_FOLD_MAX_BLOCKS / TPB;
  __shared__ int32_t s_w[2][NW];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int G = gridDim.x;
  __syncthreads();  // the block's counts are written
  const int64_t i = (int64_t)blockIdx.x * P + tid;
  const bool mine = tid < P && i < N;
  const int32_t c0 = mine ? cnt_full[i] : 0, c1 = mine ? cnt_up[i] : 0;
  int32_t s0 = c0, s1 = c1;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y0 = __shfl_up_sync(0xffffffffu, s0, o), y1 = __shfl_up_sync(0xffffffffu, s1, o);
    if (lane >= o) {
      s0 += y0;
      s1 += y1;
    }
  }
  if (lane == 31) {
    s_w[0][w] = s0;
    s_w[1][w] = s1;
  }
  __syncthreads();
  int32_t b0 = 0, b1 = 0, t0 = 0, t1 = 0;
#pragma unroll
  for (int v = 0; v < NW; ++v) {
    if (v < w) {
      b0 += s_w[0][v];
      b1 += s_w[1][v];
    }
    t0 += s_w[0][v];
    t1 += s_w[1][v];
  }
  if (mine) {
    fb[i] = b0 + s0 - c0;
    fb[N + i] = b1 + s1 - c1;
  }
  int32_t* tots = FoldRows::totals(fb, N);
  if (tid == 0) {
    tots[blockIdx.x] = t0;
    tots[G + blockIdx.x] = t1;
  }
  if (!last_block_of_grid(fold_cnt)) return;
  // the block totals' exclusive scan into the block bases (G <= ROWS_FOLD_MAX_BLOCKS)
  int32_t* bases = FoldRows::bases(fb, N, G);
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    int32_t v[IT], run = 0;
#pragma unroll
    for (int j = 0; j < IT; ++j) {
      const int idx = tid * IT + j;
      v[j] = idx < G ? __ldcg(tots + a * G + idx) : 0;
      run += v[j];
    }
    int32_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    __syncthreads();  // s_w of the pass before has been read
    if (lane == 31) s_w[a][w] = inc;
    __syncthreads();
    int32_t base = inc - run;
    for (int u = 0; u < w; ++u) base += s_w[a][u];
#pragma unroll
    for (int j = 0; j < IT; ++j) {
      const int idx = tid * IT + j;
      if (idx < G) bases[a * G + idx] = base;
      base += v[j];
    }
    if (tid == TPB - 1) {
      fb[2 * N + 4 * G + a] = base;
      (a ? rs_up : rs_full)[N] = base;
    }
  }
}

// the pair search with the FP32 prefilter (same output, same order as
// k_pairs).  MODE 4: MODE 2, then the row starts rs_full / rs_up by
// rows_fold (N + 1 <= SCAN_FOLD_MAX; a separate mode, so that the fold's
// shared memory does not weigh on MODE 2 at large N).  MODE 3: the fill, then
// the flat pair list of the pair-once passes (pairs32_quads).
template <int D, int MODE, int L>
__global__ void __launch_bounds__(TPB) k_pairs32(const double* __restrict__ x0, const double* __restrict__ x1,
                                                 const double* __restrict__ x2, const float* __restrict__ f0,
                                                 const float* __restrict__ f1, const float* __restrict__ f2,
                                                 const float2* __restrict__ thr,
                                                 const int32_t* __restrict__ skey,
                                                 const int32_t* __restrict__ cellstart, int64_t N, Grid g,
                                                 int32_t* __restrict__ cnt_full, int32_t* __restrict__ cnt_up,
                                                 const int64_t* __restrict__ rs_full, int32_t* __restrict__ nbr,
                                                 int64_t cap, int* __restrict__ ovf, int32_t* __restrict__ stg,
                                                 int S, int64_t* fold_rs_full, int64_t* fold_rs_up,
                                                 unsigned* fold_cnt, const int64_t* __restrict__ rs_up,
                                                 int4* __restrict__ pq, int32_t* fold_buf, bool up) {
  if ((MODE == 1 || MODE == 3) && fold_buf) {
    // small sets: the final row starts, from the count pass's two levels
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t k = gt / L;
    if (k < N && gt % L == 0) {
      fold_rs_full[k] = FoldRows::start(fold_buf, 0, k, N, TPB / L, gridDim.x);
      fold_rs_up[k] = FoldRows::start(fold_buf, 1, k, N, TPB / L, gridDim.x);
    }
  }
  pairs32_row<D, MODE == 3 ? 1 : (MODE == 4 ? 2 : MODE), L>(x0, x1, x2, f0, f1, f2, thr, skey, cellstart, N, g,
                                                             cnt_full, cnt_up, rs_full, nbr, cap, ovf, stg, S,
                                                             fold_buf, up);
  if (MODE == 4) rows_fold<L>(cnt_full, cnt_up, N, fold_rs_full, fold_rs_up, fold_buf, fold_cnt);
  if (MODE == 3) {
    __syncwarp();  // a recomputed row's entries, written by the group's lanes, are read back
    pairs32_quads<D, L>(N, cnt_full, cnt_up, rs_full, rs_up, nbr, cap, stg, S, pq, fold_buf);
  }
}

// lanes per particle in the pair search: about 8 candidates per lane
// Lanes per point of the pair passes.  A point walks 3^(D-1) rows of three
// cells each, and the lanes share a row's candidates, so the lanes follow the
// candidates per row: the largest power of two L at most that many, up to 32
// (measured on GB300: 16 for the 2-D dam break, 32 for 200k uniform 2-D
// points, 4 for 4M uniform 3-D points).  After a first build the candidates
// come from the mean neighbour count m = nfull / N: m times the stencil's
// volume over the dist-ball's (9/π in 2-D, 81/(4π) in 3-D, times
// (cellsize/dist)^D), which weights cells by the points in them; the first
// build takes the grid-wide mean N / ncell (which also counts empty cells).
double CellCore::candidates_per_point() const {
  if (nfull_est > 0 && N > 0) {
    double vol = D == 3 ? 81.0 / (4.0 * GCSPH_PI64) : 9.0 / GCSPH_PI64;
    for (int d = 0; d < D; ++d) vol *= cs[d] / dist;
    return (double)nfull_est / (double)N * vol;
  }
  const double per_cell = (double)N / (double)g.ncell;
  return per_cell * (D == 3 ? 27.0 : 9.0);
}

int CellCore::pair_lanes() const {
  if (lanes > 0) return lanes;
  const double cand = candidates_per_point();
  const double per_row = cand / (D == 3 ? 9.0 : 3.0);
  int L = 1;
  while (L < 32 && (double)(2 * L) <= per_row) L <<= 1;
  return L;
}

#define PAIRS_LAUNCH(MODE, L, ...)                                                               \
  do {                                                                                           \
    const int _g = nblocks(N * (int64_t)(L), TPB);                                               \
    if (D == 2) {                                                                                \
      switch (L) {                                                                               \
        case 1: k_pairs<2, MODE, 1><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                     \
        case 2: k_pairs<2, MODE, 2><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                     \
        case 4: k_pairs<2, MODE, 4><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                     \
        case 8: k_pairs<2, MODE, 8><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                     \
        case 16: k_pairs<2, MODE, 16><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        default: k_pairs<2, MODE, 32><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
      }                                                                                          \
    } else {                                                                                     \
      switch (L) {                                                                               \
        case 1: k_pairs<3, MODE, 1><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                     \
        case 2: k_pairs<3, MODE, 2><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                     \
        case 4: k_pairs<3, MODE, 4><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                     \
        case 8: k_pairs<3, MODE, 8><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                     \
        case 16: k_pairs<3, MODE, 16><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        default: k_pairs<3, MODE, 32><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
      }                                                                                          \
    }                                                                                            \
  } while (0)

#define PAIRS32_LAUNCH(MODE, L, ...)                                                             \
  do {                                                                                           \
    const int _g = nblocks(N * (int64_t)(L), TPB);                                               \
    if (D == 2) {                                                                                \
      switch (L) {                                                                               \
        case 1: k_pairs32<2, MODE, 1><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        case 2: k_pairs32<2, MODE, 2><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        case 4: k_pairs32<2, MODE, 4><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        case 8: k_pairs32<2, MODE, 8><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        case 16: k_pairs32<2, MODE, 16><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                 \
        default: k_pairs32<2, MODE, 32><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                 \
      }                                                                                          \
    } else {                                                                                     \
      switch (L) {                                                                               \
        case 1: k_pairs32<3, MODE, 1><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        case 2: k_pairs32<3, MODE, 2><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        case 4: k_pairs32<3, MODE, 4><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        case 8: k_pairs32<3, MODE, 8><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                   \
        case 16: k_pairs32<3, MODE, 16><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                 \
        default: k_pairs32<3, MODE, 32><<<_g, TPB, 0, st>>>(__VA_ARGS__); break;                 \
      }                                                                                          \
    }                                                                                            \
  } while (0)

int CellCore::ensure_pf() {
  int rc;
  for (int d = 0; d < D; ++d)
    if ((rc = pf[d].ensure(sizeof(float) * N, st))) return rc;
  if ((rc = pfthr.ensure(sizeof(float2), st))) return rc;
  if ((rc = pfcnt.ensure(sizeof(unsigned), st, true))) return rc;
  return pfmax.ensure(sizeof(unsigned long long), st, true);
}

int CellCore::build_pairs(const double* const* xs, int* ovf_dev, bool scan_up, bool pf_ready, int4* pq,
                          bool* pq_done, bool up) {
  if (pq_done) *pq_done = false;
  if (up) {
    // the half stencil: every row is its larger-index part, so both counts
    // and both row-start scans are the same; no pair list for the step
    scan_up = true;
    pq = nullptr;
  }
  if (!sorted) return fail(GCSPH_ESTATE, "pair build before binning");
  const double* x2 = D == 3 ? xs[2] : xs[0];
  timer_begin(T_PAIRS, st);
  const int L = pair_lanes();
  int rc0;
  if ((rc0 = ensure_pf())) return rc0;
  float* f2 = D == 3 ? pf[2].as<float>() : pf[0].as<float>();
  unsigned long long* bm = pfmax.as<unsigned long long>();
  float2* thr = pfthr.as<float2>();
  if (!pf_ready) {
    // (the pass's last block turns the bound into the two thresholds)
    if (D == 2)
      k_make_pf<2><<<nblocks(N, TPB), TPB, 0, st>>>(xs[0], xs[1], x2, N, g, pf[0].as<float>(), pf[1].as<float>(), f2,
                                                     bm, thr, pfcnt.as<unsigned>());
    else
      k_make_pf<3><<<nblocks(N, TPB), TPB, 0, st>>>(xs[0], xs[1], x2, N, g, pf[0].as<float>(), pf[1].as<float>(), f2,
                                                     bm, thr, pfcnt.as<unsigned>());
    GC_LAUNCHED();
  }
  // rows of up to S neighbours are staged by the count pass and copied by the fill
  // nfull_est counts full rows (a half-stencil build records twice its count)
  const double mean = N > 0 && nfull_est > 0 ? (up ? 0.5 : 1.0) * (double)nfull_est / (double)N : 0.0;
  int S = 16;
  while (S < 256 && (double)S < 1.5 * mean + 8.0) S <<= 1;
  int32_t* sp = nullptr;
  if (mean > 0 && (rc0 = stage.ensure(sizeof(int32_t) * (size_t)N * (size_t)S, st)) == GCSPH_OK) sp = stage.as<int32_t>();
  if (rc0) return rc0;
  // small sets: the count pass's last block scans the row counts (both
  // arrays), so no scan launch follows
  const bool fold = sp && foldsum.p && N + 1 <= SCAN_FOLD_MAX && nblocks(N * (int64_t)L, TPB) <= ROWS_FOLD_MAX_BLOCKS;
  unsigned* fc = fold ? foldcnt.as<unsigned>() + 1 : nullptr;
  int32_t* fbuf = fold ? foldsum.as<int32_t>() : nullptr;
  int64_t* frs_full = fold ? rs_full.as<int64_t>() : nullptr;
  int64_t* frs_up = fold ? rs_up.as<int64_t>() : nullptr;
  if (fold)
    PAIRS32_LAUNCH(4, L, xs[0], xs[1], x2, pf[0].as<float>(), pf[1].as<float>(), f2, thr, skey.as<int32_t>(),
                   cellstart.as<int32_t>(), N, g, cnt_full.as<int32_t>(), cnt_up.as<int32_t>(), nullptr, nullptr, 0,
                   nullptr, sp, S, rs_full.as<int64_t>(), rs_up.as<int64_t>(), fc, nullptr, nullptr,
                   foldsum.as<int32_t>(), up);
  else if (sp)
    PAIRS32_LAUNCH(2, L, xs[0], xs[1], x2, pf[0].as<float>(), pf[1].as<float>(), f2, thr, skey.as<int32_t>(),
                   cellstart.as<int32_t>(), N, g, cnt_full.as<int32_t>(), cnt_up.as<int32_t>(), nullptr, nullptr, 0,
                   nullptr, sp, S, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, up);
  else
    PAIRS32_LAUNCH(0, L, xs[0], xs[1], x2, pf[0].as<float>(), pf[1].as<float>(), f2, thr, skey.as<int32_t>(),
                   cellstart.as<int32_t>(), N, g, cnt_full.as<int32_t>(), cnt_up.as<int32_t>(), nullptr, nullptr, 0,
                   nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, up);
  GC_LAUNCHED();
  int rc = GCSPH_OK;
  if (!fold)
    rc = scan_up ? exclusive_scan2_i32_to_i64(cnt_full.as<int32_t>(), rs_full.as<int64_t>(), cnt_up.as<int32_t>(),
                                              rs_up.as<int64_t>(), N, scratch.as<int64_t>(), st)
                 : exclusive_scan_i32_to_i64(cnt_full.as<int32_t>(), rs_full.as<int64_t>(), N,
                                             scratch.as<int64_t>(), st);
  if (rc) return rc;
  timer_end(T_PAIRS, st);
  if (ovf_dev && nbr_cap > 0) {
    // no host round trip: fill into the current capacity; a row that would
    // pass it raises *ovf_dev, the caller's kernels then skip the step and
    // the caller grows the buffers (grow_nbr) and repeats it
    nfull = -1;
  } else {
    GC_CUDA(cudaMemcpyAsync(pin, rs_full.as<int64_t>() + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    GC_CUDA(cudaStreamSynchronize(st));
    timer_collect();
    nfull = pin[0];
    nfull_est = up ? 2 * nfull : nfull;
    if (nfull > nbr_cap && (rc = grow_nbr(nfull))) return rc;
  }
  timer_begin(T_PAIRS, st);
  if (pq && sp && scan_up && nfull < 0) {
    // the fill and the flat pair list of the pair-once passes in one launch
    // (only where the capacity did not change in this build: the caller sized
    // its pair list for it)
    PAIRS32_LAUNCH(3, L, xs[0], xs[1], x2, pf[0].as<float>(), pf[1].as<float>(), f2, thr, skey.as<int32_t>(),
                   cellstart.as<int32_t>(), N, g, cnt_full.as<int32_t>(), cnt_up.as<int32_t>(),
                   rs_full.as<int64_t>(), nbr.as<int32_t>(), nbr_cap, ovf_dev, sp, S, frs_full, frs_up, nullptr,
                   rs_up.as<int64_t>(), pq, fbuf, false);
    if (pq_done) *pq_done = true;
  } else {
    PAIRS32_LAUNCH(1, L, xs[0], xs[1], x2, pf[0].as<float>(), pf[1].as<float>(), f2, thr, skey.as<int32_t>(),
                   cellstart.as<int32_t>(), N, g, nullptr, nullptr, rs_full.as<int64_t>(), nbr.as<int32_t>(), nbr_cap,
                   ovf_dev, sp, S, frs_full, frs_up, nullptr, nullptr, nullptr, fbuf, up);
  }
  GC_LAUNCHED();
  timer_end(T_PAIRS, st);
  built = true;
  up_valid = false;
  rows_upper = up;
  return GCSPH_OK;
}

int CellCore::grow_nbr(int64_t need) {
  const int64_t want = need + need / 4 + 1024;
  int rc = nbr.ensure(sizeof(int32_t) * want, st);
  if (rc) return rc;
  nbr_cap = want;
  gen += 1;
  return GCSPH_OK;
}

int CellCore::read_nfull() {
  GC_CUDA(cudaMemcpyAsync(pin, rs_full.as<int64_t>() + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GC_CUDA(cudaStreamSynchronize(st));
  nfull = pin[0];
  nfull_est = rows_upper ? 2 * nfull : nfull;
  return GCSPH_OK;
}

// offsets of each sorted particle's pairs in the (min,max) list: scanned on
// demand, the stepping loop never needs them
int CellCore::ensure_up() {
  if (up_valid) return GCSPH_OK;
  int rc = exclusive_scan_i32_to_i64(cnt_up.as<int32_t>(), rs_up.as<int64_t>(), N, scratch.as<int64_t>(), st);
  if (rc) return rc;
  GC_CUDA(cudaMemcpyAsync(pin + 1, rs_up.as<int64_t>() + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GC_CUDA(cudaStreamSynchronize(st));
  nup = pin[1];
  up_valid = true;
  return GCSPH_OK;
}

int CellCore::emit(int32_t* pairs, int64_t cap, int fillzero, int64_t* pairsn) {
  if (!built) return fail(GCSPH_ESTATE, "no pair set built yet");
  if (cap < 0) return fail(GCSPH_EINVAL, "negative capacity");
  int rc0 = ensure_up();
  if (rc0) return rc0;
  if (pairsn) *pairsn = nup;
  if (cap > 0 && !pairs) return fail(GCSPH_EINVAL, "null pair buffer");
  if (cap > 0) {
    if (((uintptr_t)pairs & 7u) == 0) {
      // lanes per point: about four pairs each, from the mean upper row
      const double mean = N > 0 ? (double)nup / (double)N : 0.0;
      int L = 1;
      while (L < 32 && (double)L * 4.0 < mean) L <<= 1;
      const int g = nblocks(N * (int64_t)L, TPB);
      int2* p2 = reinterpret_cast<int2*>(pairs);
      const int64_t* rf = rs_full.as<int64_t>();
      const int64_t* ru = rs_up.as<int64_t>();
      const int32_t* nb = nbr.as<int32_t>();
      const int32_t* og = orig.as<int32_t>();
      switch (L) {
        case 1: k_emit_pairs_l<1><<<g, TPB, 0, st>>>(rf, ru, nb, og, N, cap, p2); break;
        case 2: k_emit_pairs_l<2><<<g, TPB, 0, st>>>(rf, ru, nb, og, N, cap, p2); break;
        case 4: k_emit_pairs_l<4><<<g, TPB, 0, st>>>(rf, ru, nb, og, N, cap, p2); break;
        case 8: k_emit_pairs_l<8><<<g, TPB, 0, st>>>(rf, ru, nb, og, N, cap, p2); break;
        case 16: k_emit_pairs_l<16><<<g, TPB, 0, st>>>(rf, ru, nb, og, N, cap, p2); break;
        default: k_emit_pairs_l<32><<<g, TPB, 0, st>>>(rf, ru, nb, og, N, cap, p2); break;
      }
    } else {
      k_emit_pairs<<<nblocks(N, TPB), TPB, 0, st>>>(rs_full.as<int64_t>(), rs_up.as<int64_t>(), nbr.as<int32_t>(),
                                                     orig.as<int32_t>(), N, cap, pairs);
    }
    GC_LAUNCHED();
    if (fillzero && nup < cap)
      GC_CUDA(cudaMemsetAsync(pairs + 2 * nup, 0, sizeof(int32_t) * 2 * (size_t)(cap - nup), st));
  }
  GC_CUDA(cudaStreamSynchronize(st));
  if (nup > cap) return fail(GCSPH_ECAPACITY, "pair list holds %lld of %lld pairs", (long long)cap, (long long)nup);
  return GCSPH_OK;
}

int CellCore::maxpairs(int64_t* out) {
  int64_t* d = scratch.as<int64_t>();
  GC_CUDA(cudaMemsetAsync(d, 0, sizeof(int64_t), st));
  if (D == 2)
    k_maxpairs<2><<<nblocks(g.ncell, TPB), TPB, 0, st>>>(cellstart.as<int32_t>(), g, (unsigned long long*)d);
  else
    k_maxpairs<3><<<nblocks(g.ncell, TPB), TPB, 0, st>>>(cellstart.as<int32_t>(), g, (unsigned long long*)d);
  GC_LAUNCHED();
  return read_scalar(d, out);
}

}  // namespace gcsph

// ---------------------------------------------------------------------------
// C ABI: gcl_*
// ---------------------------------------------------------------------------
using namespace gcsph;

// update! and partialupdate! return the pairs k < m only: their builds take
// the half stencil
static int gcl_full_update(gcl_handle* h) {
  int rc = h->core.sort(h->xuser, nullptr, true);
  if (rc) return rc;
  double* xs[3] = {h->xs[0].as<double>(), h->xs[1].as<double>(), h->core.D == 3 ? h->xs[2].as<double>() : nullptr};
  if ((rc = h->core.gather_positions(h->xuser, xs))) return rc;
  return h->core.build_pairs((const double* const*)xs, nullptr, false, false, nullptr, nullptr, true);
}

extern "C" {

int gcl_create(int32_t D, int64_t N, const double* const* x_dev, const double* cellsize, double dist,
               const double* MIN_or_null, const double* MAX_or_null, void* stream, gcl_handle** out) {
  if (!out || !x_dev || !cellsize) return fail(GCSPH_EINVAL, "null argument");
  *out = nullptr;
  if (D != 2 && D != 3) return fail(GCSPH_EINVAL, "wrong dimention: D=%d (2 or 3)", (int)D);
  for (int d = 0; d < D; ++d)
    if (!x_dev[d]) return fail(GCSPH_EINVAL, "null coordinate array %d", d + 1);
  gcl_handle* h = new gcl_handle();
  for (int d = 0; d < D; ++d) h->xuser[d] = x_dev[d];
  int rc = h->core.init(D, N, cellsize, dist, MIN_or_null, MAX_or_null, x_dev, (cudaStream_t)stream);
  if (!rc)
    for (int d = 0; d < D && !rc; ++d) rc = h->xs[d].ensure(sizeof(double) * N, h->core.st);
  if (!rc) rc = gcl_full_update(h);
  if (rc) {
    std::string keep = gcsph_last_error();
    h->core.release();
    for (auto& b : h->xs) b.release();
    delete h;
    set_error("%s", keep.c_str());
    return rc;
  }
  *out = h;
  return GCSPH_OK;
}

void gcl_destroy(gcl_handle* h) {
  if (!h) return;
  cudaStreamSynchronize(h->core.st);
  h->core.release();
  for (auto& b : h->xs) b.release();
  delete h;
}

int gcl_grid(const gcl_handle* h, double* cs, double* offset, int64_t* cell) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  for (int d = 0; d < h->core.D; ++d) {
    if (cs) cs[d] = h->core.cs[d];
    if (offset) offset[d] = h->core.g.offset[d];
    if (cell) cell[d] = h->core.g.nc[d];
  }
  return GCSPH_OK;
}

int gcl_update(gcl_handle* h, int64_t* pairsn_out) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  int rc = gcl_full_update(h);
  if (rc) return rc;
  if ((rc = h->core.ensure_up())) return rc;
  if (pairsn_out) *pairsn_out = h->core.nup;
  GC_CUDA(cudaStreamSynchronize(h->core.st));
  return GCSPH_OK;
}

int gcl_partialupdate(gcl_handle* h, int64_t* pairsn_out) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  if (!h->core.sorted) return fail(GCSPH_ESTATE, "partialupdate before any update");
  double* xs[3] = {h->xs[0].as<double>(), h->xs[1].as<double>(), h->core.D == 3 ? h->xs[2].as<double>() : nullptr};
  int rc = h->core.gather_positions_by_orig(h->xuser, xs);
  if (rc) return rc;
  if ((rc = h->core.build_pairs((const double* const*)xs, nullptr, false, false, nullptr, nullptr, true))) return rc;
  if ((rc = h->core.ensure_up())) return rc;
  if (pairsn_out) *pairsn_out = h->core.nup;
  GC_CUDA(cudaStreamSynchronize(h->core.st));
  return GCSPH_OK;
}

int gcl_emit_pairs(gcl_handle* h, int32_t* pairs_dev, int64_t cap, int fillzero, int64_t* pairsn_out) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  return h->core.emit(pairs_dev, cap, fillzero, pairsn_out);
}

int gcl_cellpnum(gcl_handle* h, int32_t* cellpnum_dev) {
  if (!h || !cellpnum_dev) return fail(GCSPH_EINVAL, "null argument");
  const int64_t nc = h->core.g.ncell;
  k_cell_pop<<<nblocks(nc, TPB), TPB, 0, h->core.st>>>(h->core.cellstart.as<int32_t>(), nc, cellpnum_dev);
  GC_LAUNCHED();
  GC_CUDA(cudaStreamSynchronize(h->core.st));
  return GCSPH_OK;
}

int gcl_maxpairs(gcl_handle* h, int64_t* out) {
  if (!h || !out) return fail(GCSPH_EINVAL, "null argument");
  return h->core.maxpairs(out);
}

int gcl_set_sort(gcl_handle* h, int32_t mode) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  if (mode < 0 || mode > 2) return fail(GCSPH_EINVAL, "sort mode %d (0, 1 or 2)", (int)mode);
  h->core.sort_mode = mode;
  return GCSPH_OK;
}

}  // extern "C"

// ===========================================================================
// gcl_pairs_noalloc: GPUCellList + neighborlist in one call that allocates no
// memory.  For callers that may not allocate device memory while they run --
// a host whose own memory pool already holds the device (a Julia or PyTorch
// process that reserved it), a plugin whose framework forbids allocation, or
// a time-critical loop that cannot absorb cudaMalloc's implicit device
// synchronisation.  Every intermediate array lives in one file-scope
// __device__ arena sized for GCSPH_NOALLOC_MAX_POINTS points and
// GCSPH_NOALLOC_MAX_CELLS grid cells; each GPU that loads this library keeps
// that arena (24 MiB) until the process exits.  The caller passes the
// coordinates and owns the output pair buffer.  CUDA reserves the arena when
// it loads this file's module, which under lazy module loading happens at
// the first use, so gcl_pairs_noalloc_init (or a first call) must come
// before the caller's own pool takes the device's memory.
// ===========================================================================
namespace gcsph {
namespace noalloc {

constexpr int64_t MAXN = GCSPH_NOALLOC_MAX_POINTS;
constexpr int64_t MAXC = GCSPH_NOALLOC_MAX_CELLS;
constexpr int64_t al(int64_t b) { return (b + 255) / 256 * 256; }
// arena layout, byte offsets
constexpr int64_t O_KEY = 0;
constexpr int64_t O_SLOT = O_KEY + al(4 * MAXN);
constexpr int64_t O_TMP = O_SLOT + al(4 * MAXN);
constexpr int64_t O_PERM = O_TMP + al(4 * MAXN);
constexpr int64_t O_SKEY = O_PERM + al(4 * MAXN);
constexpr int64_t O_ORIG = O_SKEY + al(4 * MAXN);
constexpr int64_t O_XS = O_ORIG + al(4 * MAXN);
constexpr int64_t O_COUNT = O_XS + al(3 * 8 * MAXN);
constexpr int64_t O_CSTART = O_COUNT + al(4 * MAXC);
constexpr int64_t O_CFULL = O_CSTART + al(4 * (MAXC + 1));
constexpr int64_t O_CUP = O_CFULL + al(4 * MAXN);
constexpr int64_t O_RSUP = O_CUP + al(4 * MAXN);
constexpr int64_t O_SCAN = O_RSUP + al(8 * (MAXN + 1));
// the device scan's scratch, sized by the scan's own rule for the longer of
// the two scans (ncell + 1 and N + 1 items)
constexpr int64_t O_MINMAX = O_SCAN + al(8 * scan_scratch_elems((MAXC > MAXN ? MAXC : MAXN) + 1));
constexpr int64_t BYTES = O_MINMAX + al(8 * 2 * 3 * MINMAX_MAX_BLOCKS);

}  // namespace noalloc
}  // namespace gcsph

// the scratch of gcl_pairs_noalloc; host code must not use this name as a
// device address -- it reaches the kernels through cudaGetSymbolAddress
static __device__ __align__(256) unsigned char g_noalloc_arena[gcsph::noalloc::BYTES];

namespace gcsph {
namespace noalloc {

// fill pass that writes the (min,max) 1-based pairs of each sorted particle's
// larger-index neighbours straight into the caller's list, ascending, at the
// scanned offset: the same list gcl_emit_pairs writes from the neighbour CSR
template <int D, int L>
__global__ void __launch_bounds__(TPB) k_pairs_direct(const double* __restrict__ x0, const double* __restrict__ x1,
                                                      const double* __restrict__ x2, const int32_t* __restrict__ skey,
                                                      const int32_t* __restrict__ cellstart,
                                                      const int32_t* __restrict__ orig, int64_t N, Grid g,
                                                      const int64_t* __restrict__ rs_up, int64_t cap,
                                                      int32_t* __restrict__ pairs) {
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;
  const unsigned lanew = threadIdx.x & 31u;
  const unsigned gbase = lanew & ~(unsigned)(L - 1);
  const unsigned gm = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << gbase);
  const int nx = g.nc[0], ny = g.nc[1], nz = D == 3 ? g.nc[2] : 1;
  const int32_t key = skey[k];
  const int cx = key % nx;
  const int t = key / nx;
  const int cy = t % ny;
  const int cz = t / ny;
  const double ax = x0[k], ay = x1[k], az = D == 3 ? x2[k] : 0.0;
  const int32_t ok = orig[k] + 1;
  int64_t wpos = rs_up[k];
  const int xlo = cx > 0 ? cx - 1 : 0;
  const int xhi = cx < nx - 1 ? cx + 1 : nx - 1;
  for (int dz = (D == 3 ? -1 : 0); dz <= (D == 3 ? 1 : 0); ++dz) {
    const int z = cz + dz;
    if (z < 0 || z >= nz) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= ny) continue;
      const int64_t base = (int64_t)nx * ((int64_t)y + (int64_t)ny * z);
      const int32_t m0 = cellstart[base + xlo], m1 = cellstart[base + xhi + 1];
      for (int32_t mb = m0; mb < m1; mb += L) {
        const int32_t m = mb + lane;
        bool hit = false;
        if (m < m1 && m > k) hit = r2_ref<D>(ax, ay, az, x0[m], x1[m], D == 3 ? x2[m] : 0.0) < g.dist2;
        const unsigned bal = (__ballot_sync(gm, hit) >> gbase) & (L == 32 ? 0xffffffffu : ((1u << L) - 1u));
        if (hit) {
          const int64_t pos = wpos + __popc(bal & ((1u << lane) - 1u));
          if (pos < cap) {
            const int32_t om = orig[m] + 1;
            pairs[2 * pos] = ok < om ? ok : om;
            pairs[2 * pos + 1] = ok < om ? om : ok;
          }
        }
        wpos += __popc(bal);
      }
    }
  }
}

static std::mutex g_mu;
static void* g_arena_of[128] = {nullptr};
static int g_minmax_blocks_of[128] = {0};

// every kernel a call can launch, loaded into the current context now: with
// lazy module loading (the CUDA default) each is otherwise loaded at its
// first launch, which takes device memory for its code
template <int D>
static int preload_dim() {
  cudaFuncAttributes a;
  const void* fns[] = {(const void*)k_cellkey<D>,           (const void*)k_gather_pos<D>,
                       (const void*)k_pairs<D, 0, 1>,       (const void*)k_pairs<D, 0, 2>,
                       (const void*)k_pairs<D, 0, 4>,       (const void*)k_pairs<D, 0, 8>,
                       (const void*)k_pairs<D, 0, 16>,      (const void*)k_pairs<D, 0, 32>,
                       (const void*)k_pairs_direct<D, 1>,   (const void*)k_pairs_direct<D, 2>,
                       (const void*)k_pairs_direct<D, 4>,   (const void*)k_pairs_direct<D, 8>,
                       (const void*)k_pairs_direct<D, 16>,  (const void*)k_pairs_direct<D, 32>};
  for (const void* f : fns) GC_CUDA(cudaFuncGetAttributes(&a, f));
  return GCSPH_OK;
}

// device address of the arena on the current device, and this device's
// bounding-box grid; set up once per device, with the device's kernels
// loaded at the same time
static int arena(unsigned char** out, int* minmax_nb) {
  int dev = 0;
  GC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return fail(GCSPH_EINVAL, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_arena_of[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_arena);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_arena)", __FILE__, __LINE__);
    cudaFuncAttributes a;
    const void* fns[] = {(const void*)k_minmax, (const void*)k_scatter_arrival, (const void*)k_rank_in_cell,
                         (const void*)k_apply_perm};
    for (const void* f : fns) GC_CUDA(cudaFuncGetAttributes(&a, f));
    int rc = preload_dim<2>();
    if (!rc) rc = preload_dim<3>();
    if (!rc) rc = scan_preload();
    if (rc) return rc;
    g_minmax_blocks_of[dev] = minmax_blocks();
    g_arena_of[dev] = p;
  }
  *out = (unsigned char*)g_arena_of[dev];
  if (minmax_nb) *minmax_nb = g_minmax_blocks_of[dev];
  return GCSPH_OK;
}

template <int D>
static int run(int64_t N, const double* const* x, const double* cellsize, double dist, const double* MIN,
               const double* MAX, int32_t* pairs, int64_t cap, int fillzero, int64_t* pairsn, cudaStream_t st) {
  unsigned char* A = nullptr;
  int nb = 0;
  int rc = arena(&A, &nb);
  if (rc) return rc;
  int32_t* key = (int32_t*)(A + O_KEY);
  int32_t* slot = (int32_t*)(A + O_SLOT);
  int32_t* tmpv = (int32_t*)(A + O_TMP);
  int32_t* perm = (int32_t*)(A + O_PERM);
  int32_t* skey = (int32_t*)(A + O_SKEY);
  int32_t* orig = (int32_t*)(A + O_ORIG);
  double* xs[3] = {(double*)(A + O_XS), (double*)(A + O_XS) + MAXN, (double*)(A + O_XS) + 2 * MAXN};
  int32_t* count = (int32_t*)(A + O_COUNT);
  int32_t* cstart = (int32_t*)(A + O_CSTART);
  int32_t* cfull = (int32_t*)(A + O_CFULL);
  int32_t* cup = (int32_t*)(A + O_CUP);
  int64_t* rsup = (int64_t*)(A + O_RSUP);
  int64_t* scan = (int64_t*)(A + O_SCAN);
  double* mm = (double*)(A + O_MINMAX);
  // frozen grid, src/celllist.jl:27-46
  const double seps = 1.4901161193847656e-08;  // sqrt(eps(Float64)) = 2^-26
  Grid g{};
  int64_t ncell = 1;
  double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
  if (!MIN || !MAX) {
    // pageable host copy of the per-block partials, on the stack (48 KB)
    double host[2 * 3 * MINMAX_MAX_BLOCKS];
    if ((rc = bounding_box(D, x, N, nb, mm, host, st, bmin, bmax))) return rc;
  }
  for (int d = 0; d < D; ++d) {
    double lo = MIN ? MIN[d] : bmin[d];
    double hi = MAX ? MAX[d] : bmax[d];
    const double cs = cellsize[d] < dist ? dist : cellsize[d];
    lo = lo - fabs((lo + seps) * seps);
    const double c = ceil((hi - lo) / cs);
    if (!(c >= 1.0) || c > 2.0e9) return fail(GCSPH_EINVAL, "degenerate grid in dim %d (CELL=%g)", d + 1, c);
    g.offset[d] = lo;
    g.hinv[d] = 1.0 / cs;
    g.nc[d] = (int)c;
    ncell *= (int64_t)c;
    if (ncell > MAXC)
      return fail(GCSPH_EINVAL,
                  "gcl_pairs_noalloc: the cell grid needs more than %lld cells, the limit of its static scratch "
                  "(use gcl_create for larger grids)",
                  (long long)MAXC);
  }
  for (int d = D; d < 3; ++d) g.nc[d] = 1;
  g.D = D;
  g.ncell = ncell;
  g.dist2 = dist * dist;
  // binning and counting sort; the arena keeps the previous call's contents,
  // so the per-cell counters are cleared first
  GC_CUDA(cudaMemsetAsync(count, 0, sizeof(int32_t) * ncell, st));
  const double* x2 = D == 3 ? x[2] : x[0];
  k_cellkey<D><<<nblocks(N, TPB), TPB, 0, st>>>(x[0], x[1], x2, N, g, key, slot, count, nullptr, nullptr, nullptr);
  GC_LAUNCHED();
  if ((rc = exclusive_scan_i32_to_i32(count, cstart, ncell, scan, st))) return rc;
  k_scatter_arrival<<<nblocks(N, TPB), TPB, 0, st>>>(key, slot, cstart, N, tmpv);
  GC_LAUNCHED();
  k_rank_in_cell<<<nblocks(N, TPB), TPB, 0, st>>>(tmpv, key, cstart, nullptr, N, perm);
  GC_LAUNCHED();
  k_apply_perm<<<nblocks(N, TPB), TPB, 0, st>>>(perm, key, nullptr, N, skey, orig);
  GC_LAUNCHED();
  k_gather_pos<D><<<nblocks(N, TPB), TPB, 0, st>>>(perm, N, x[0], x[1], x2, xs[0], xs[1], D == 3 ? xs[2] : nullptr);
  GC_LAUNCHED();
  // pair counts, offsets, then the pairs themselves
  const double cand = (double)N / (double)ncell * (D == 3 ? 27.0 : 9.0);
  int L = 1;
  while (L < 32 && (double)L * 8.0 < cand) L <<= 1;
  const double* xc2 = D == 3 ? xs[2] : xs[0];
  const int gb = nblocks(N * (int64_t)L, TPB);
#define NA_CASES(KER, ...)                                              \
  switch (L) {                                                          \
    case 1: KER<D, 1><<<gb, TPB, 0, st>>>(__VA_ARGS__); break;          \
    case 2: KER<D, 2><<<gb, TPB, 0, st>>>(__VA_ARGS__); break;          \
    case 4: KER<D, 4><<<gb, TPB, 0, st>>>(__VA_ARGS__); break;          \
    case 8: KER<D, 8><<<gb, TPB, 0, st>>>(__VA_ARGS__); break;          \
    case 16: KER<D, 16><<<gb, TPB, 0, st>>>(__VA_ARGS__); break;        \
    default: KER<D, 32><<<gb, TPB, 0, st>>>(__VA_ARGS__); break;        \
  }
  switch (L) {
    case 1: k_pairs<D, 0, 1><<<gb, TPB, 0, st>>>(xs[0], xs[1], xc2, skey, cstart, N, g, cfull, cup, nullptr, nullptr); break;
    case 2: k_pairs<D, 0, 2><<<gb, TPB, 0, st>>>(xs[0], xs[1], xc2, skey, cstart, N, g, cfull, cup, nullptr, nullptr); break;
    case 4: k_pairs<D, 0, 4><<<gb, TPB, 0, st>>>(xs[0], xs[1], xc2, skey, cstart, N, g, cfull, cup, nullptr, nullptr); break;
    case 8: k_pairs<D, 0, 8><<<gb, TPB, 0, st>>>(xs[0], xs[1], xc2, skey, cstart, N, g, cfull, cup, nullptr, nullptr); break;
    case 16: k_pairs<D, 0, 16><<<gb, TPB, 0, st>>>(xs[0], xs[1], xc2, skey, cstart, N, g, cfull, cup, nullptr, nullptr); break;
    default: k_pairs<D, 0, 32><<<gb, TPB, 0, st>>>(xs[0], xs[1], xc2, skey, cstart, N, g, cfull, cup, nullptr, nullptr); break;
  }
  GC_LAUNCHED();
  if ((rc = exclusive_scan_i32_to_i64(cup, rsup, N, scan, st))) return rc;
  int64_t total = 0;
  GC_CUDA(cudaMemcpyAsync(&total, rsup + N, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GC_CUDA(cudaStreamSynchronize(st));
  if (cap > 0) {
    NA_CASES(k_pairs_direct, xs[0], xs[1], xc2, skey, cstart, orig, N, g, rsup, cap, pairs);
    GC_LAUNCHED();
    if (fillzero && total < cap)
      GC_CUDA(cudaMemsetAsync(pairs + 2 * total, 0, sizeof(int32_t) * 2 * (size_t)(cap - total), st));
  }
#undef NA_CASES
  GC_CUDA(cudaStreamSynchronize(st));
  if (pairsn) *pairsn = total;
  if (total > cap)
    return fail(GCSPH_ECAPACITY, "pair list holds %lld of %lld pairs", (long long)cap, (long long)total);
  return GCSPH_OK;
}

}  // namespace noalloc
}  // namespace gcsph

extern "C" int gcl_pairs_noalloc(int32_t D, int64_t N, const double* const* x_dev, const double* cellsize,
                                 double dist, const double* MIN_or_null, const double* MAX_or_null,
                                 int32_t* pairs_dev, int64_t cap, int fillzero, int64_t* pairsn_out, void* stream) {
  using namespace gcsph;
  if (!x_dev || !cellsize) return fail(GCSPH_EINVAL, "null argument");
  if (D != 2 && D != 3) return fail(GCSPH_EINVAL, "wrong dimention: D=%d (2 or 3)", (int)D);
  for (int d = 0; d < D; ++d)
    if (!x_dev[d]) return fail(GCSPH_EINVAL, "null coordinate array %d", d + 1);
  if (N < 1) return fail(GCSPH_EINVAL, "N=%lld out of range", (long long)N);
  if (N > noalloc::MAXN)
    return fail(GCSPH_EINVAL,
                "gcl_pairs_noalloc: %lld points exceed the limit of its static scratch, %lld "
                "(use gcl_create for larger sets)",
                (long long)N, (long long)noalloc::MAXN);
  if (!(dist > 0)) return fail(GCSPH_EINVAL, "dist must be > 0");
  if (cap < 0 || (cap > 0 && !pairs_dev)) return fail(GCSPH_EINVAL, "bad pair buffer");
  cudaStream_t st = (cudaStream_t)stream;
  return D == 2 ? noalloc::run<2>(N, x_dev, cellsize, dist, MIN_or_null, MAX_or_null, pairs_dev, cap, fillzero,
                                  pairsn_out, st)
                : noalloc::run<3>(N, x_dev, cellsize, dist, MIN_or_null, MAX_or_null, pairs_dev, cap, fillzero,
                                  pairsn_out, st);
}

extern "C" int gcl_pairs_noalloc_init(void) {
  unsigned char* A = nullptr;
  return gcsph::noalloc::arena(&A, nullptr);
}
