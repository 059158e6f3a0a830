// celllist.cuh -- cell binning + pair-set build shared by gcl_* and sph_*.
//
// HBM layout (all device, one handle):
//   key[N], slot[N]     cell key and arrival slot of each particle in input order
//   count[ncell]        particles per cell (= the reference's cellpnum)
//   cellstart[ncell+1]  exclusive scan of count
//   tmp[N]              arrival-ordered members of each cell
//   perm[N]             sorted position -> input index; cells ascending, and
//                       inside a cell ascending ORIGINAL particle index
//   skey[N], orig[N]    cell key and original index of each sorted particle
//   rs_full[N+1], nbr[] CSR of every neighbour (both directions) of each sorted
//                       particle, neighbours ascending -- the fused SPH sums walk it
//   rs_up[N+1]          per-particle count of neighbours with a larger sorted
//                       index, scanned -- position of that particle's pairs in
//                       the emitted (min,max) pair list
#pragma once
#include "gcsph_common.cuh"

namespace gcsph {

struct Grid {
  int D;
  double offset[3];
  double hinv[3];
  int nc[3];
  int64_t ncell;
  double dist2;
};

// the cell of point i (0-based linear key, x fastest): kernel_cellmap!'s
// clamped ceil((x - offset) / cellsize), src/gpukernels_cls.jl:28-60
template <int D>
__device__ inline int32_t cell_key_v(const double* xv, const Grid& g) {
  int64_t lin = 0, stride = 1;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double p = (xv[d] - g.offset[d]) * g.hinv[d];
    const double c = fmin(fmax(p, 1.0), (double)g.nc[d]);
    const int ci = (int)ceil(c);
    lin += (int64_t)(ci - 1) * stride;
    stride *= g.nc[d];
  }
  return (int32_t)lin;
}
template <int D>
__device__ inline int32_t cell_key(const double* x0, const double* x1, const double* x2, int64_t i, const Grid& g) {
  double xv[3] = {x0[i], x1[i], D == 3 ? x2[i] : 0.0};
  return cell_key_v<D>(xv, g);
}

// The counting sort's last step for the point in arrival position q: its
// rank among its cell's points by original index (a stable, history-free
// order; cost: the cell's population), and so its slot k in cell order,
// where the map entries go.  Returns k; *i_out is the point's input index.
// With tord (the order value of each arrival-list entry, written beside tmp)
// the cell's values are one contiguous run, read without a second, dependent
// load per member.
__device__ inline int64_t rank_in_cell(const int32_t* __restrict__ tmp, const int32_t* __restrict__ key,
                                       const int32_t* __restrict__ cellstart, const int32_t* __restrict__ ord,
                                       int64_t q, int32_t* __restrict__ perm, int32_t* __restrict__ skey,
                                       int32_t* __restrict__ orig, int32_t* i_out = nullptr,
                                       const int32_t* __restrict__ tord = nullptr) {
  const int32_t i = tmp[q];
  const int32_t c = key[i];
  const int32_t s = cellstart[c], e = cellstart[c + 1];
  int32_t r = 0;
  int32_t oi;
  if (tord) {
    oi = tord[q];
#pragma unroll 4
    for (int32_t t = s; t < e; ++t) r += (tord[t] < oi);
  } else {
    oi = ord ? ord[i] : i;
    for (int32_t t = s; t < e; ++t) {
      const int32_t j = tmp[t];
      const int32_t oj = ord ? ord[j] : j;
      r += (oj < oi);
    }
  }
  perm[s + r] = i;
  skey[s + r] = c;
  orig[s + r] = oi;
  if (i_out) *i_out = i;
  return s + r;
}

template <int D>
__device__ inline void pf_thresholds_from(unsigned long long bits, double dist2, float* tlo, float* thi) {
  const double B = __longlong_as_double((long long)bits) * (1.0 + 0x1p-28);
  const double e0 = B * 0x1p-22;
  const double Tp = 1.5 * dist2;
  const double band = 2.0 * e0 * sqrt((double)D * Tp) + (double)D * e0 * e0 + Tp * 0x1p-20;
  *tlo = __double2float_rd(dist2 - band);
  *thi = __double2float_ru(dist2 + band);
}

// The pass that accumulates the bound (max |x - offset|, atomically, per
// warp) ends with this, every thread of every block: the last block to
// finish turns the bound into the two thresholds and resets the counter.
template <int D>
__device__ inline void pf_thresholds_last_block(unsigned long long* bmax, double dist2, float2* thr, unsigned* cnt) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(cnt, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    float lo, hi;
    pf_thresholds_from<D>(atomicAdd(bmax, 0ull), dist2, &lo, &hi);
    *thr = make_float2(lo, hi);
    *cnt = 0u;
  }
}

// bounding box of D coordinate arrays (celllist.jl:41-43) with one launch
// of nb blocks per dimension and one wait; a NaN coordinate is refused with
// GCSPH_EINVAL.  part_dev and part_host hold 2 * D * nb doubles.
constexpr int MINMAX_MAX_BLOCKS = 1024;
int minmax_blocks();
int bounding_box(int D, const double* const* x, int64_t N, int nb, double* part_dev, double* part_host,
                 cudaStream_t st, double* mn, double* mx);

// sets of more points than this are ordered by the stable radix sort (O(N));
// smaller ones by the counting sort's in-cell rank (fewer launches)
constexpr int64_t RADIX_MIN_N = 65536;
// ... and then only where a cell holds more than this many points (below it
// the rank's cost is a few loads per point and takes fewer launches)
constexpr int RADIX_MIN_POP = 128;
// blocks of the count pass whose row-start scan it folds (rows_fold)
constexpr int ROWS_FOLD_MAX_BLOCKS = 2048;

struct CellCore {
  int D = 2;
  int64_t N = 0;
  double dist = 0, cs[3] = {0, 0, 0};
  Grid g{};
  cudaStream_t st = 0;

  // count (points per cell) is a binning's scratch and zero at rest: each
  // binning zeroes it again once scanned; a cell's population is
  // cellstart[c + 1] - cellstart[c]
  DevBuf count, cellstart, key, slot, tmp, perm, skey, orig, orig_b, cnt_full, cnt_up, rs_full, rs_up, nbr, scratch;
  DevBuf tord;          // the arrival lists' order values (ord of each tmp entry): the rank reads one array
  DevBuf pf[3], pfmax;  // FP32 (x - offset) copies for the prefilter, and max |x - offset|
  DevBuf pfthr;         // the prefilter's two FP32 thresholds (float2), from pfmax once per build
  DevBuf pfcnt;         // blocks done of the pass that accumulates pfmax (its last block writes pfthr)
  DevBuf stage;         // neighbour rows staged by the count pass (fixed stride), copied by the fill
  DevBuf foldcnt;       // finished-block counters of the passes whose last block runs a scan (2 unsigned)
  DevBuf foldsum;       // block totals of the folded row-start scan (small sets)
  DevBuf rkey[2], rval[2], rhist, rhoff;  // radix sort of large sets: ping-pong keys/values, tile histograms
  int64_t* pin = nullptr;  // pinned host scalars
  int64_t nfull = 0, nup = 0, nbr_cap = 0;
  int64_t nfull_est = 0;  // last neighbour-entry count read back (lane choice); nfull is -1 while unknown
  int64_t gen = 0;        // bumped whenever a buffer a captured step graph points into is reallocated
  bool sorted = false, built = false, up_valid = false;
  bool rows_upper = false;  // the last build stored the larger-index part of each row only
  int lanes = 0;  // lanes per particle in the pair search; 0 = by mean candidate count
  int sort_mode = 0;    // in-cell order: 0 by the population, 1 counting sort's rank, 2 radix sort
  int last_popmax = 0;  // largest cell population seen (large sets; read where the host waits anyway)
  DevBuf popmax;
  int pair_lanes() const;
  // candidates (points in the 3^D stencil) per point: from the last build's
  // neighbour count, else from the grid-wide mean per cell
  double candidates_per_point() const;

  int init(int D_, int64_t N_, const double* cellsize, double dist_, const double* MIN, const double* MAX,
           const double* const* xin, cudaStream_t s);
  void release();
  // bin xin (input order) into the frozen grid and sort by (cell, ord[i]);
  // ord == nullptr means the input order is the original order.
  // may_sync: the caller waits anyway, so the most crowded cell of this very
  // binning is read back to pick the ordering (else the last one read)
  // rank_deferred (the counting sort's path only, where it is set true):
  // stop after the arrival lists; the caller ranks each point with
  // rank_in_cell in a pass of its own and then calls sort_done
  // keys_ready: the cell keys, arrival slots and cell starts of xin were
  // written by the step's last pass (small sets whose cell starts that pass
  // scans, see keys_in_step), so the binning starts at the arrival lists
  int sort(const double* const* xin, const int32_t* ord, bool may_sync = false, bool* rank_deferred = nullptr,
           bool keys_ready = false);
  // whether the next binning's keys may come from the step's last pass: a
  // grid whose cell starts one block scans, and the counting sort's order
  bool keys_in_step() const { return g.ncell + 1 <= SCAN_FOLD_MAX && N <= RADIX_MIN_N && sort_mode != 2; }
  // the bookkeeping after a binning into perm / skey / orig_b (orig_b becomes orig)
  void sort_done();
  int read_popmax();
  // gather xs[d][k] = xin[d][perm[k]] (and orig[k] = ord[perm[k]] is done by sort)
  int gather_positions(const double* const* xin, double* const* xs);
  // gather xs[d][k] = xorig[d][orig[k]] for partial updates
  int gather_positions_by_orig(const double* const* xorig, double* const* xs);
  // count + scan + fill of the neighbour CSR on sorted positions xs.  With
  // ovf_dev (and buffers already sized once) the fill does not wait for the
  // count: rows past nbr_cap raise *ovf_dev instead (see grow_nbr).  scan_up
  // also scans the larger-index counts into rs_up (device only) in the same
  // launch as the row offsets.
  // pf_ready: the FP32 prefilter copy of xs (pf, pfmax) was written by the caller's permute.
  // pq (with scan_up): the fill also writes the flat pair list (k, m, e, mirror(e)) of the
  // pair-once passes when the count pass staged the rows and the fill runs without a host
  // round trip (the capacity unchanged: pq must hold nbr_cap / 2 + 1 pairs); *pq_done says
  // whether it did
  // up: the half stencil (only the m > k part of each row is searched and
  // stored: rs_full == rs_up), for callers that need the pairs k < m alone
  int build_pairs(const double* const* xs, int* ovf_dev = nullptr, bool scan_up = false, bool pf_ready = false,
                  int4* pq = nullptr, bool* pq_done = nullptr, bool up = false);
  int ensure_pf();
  int grow_nbr(int64_t need);
  int read_nfull();
  int ensure_up();
  // (min,max) 1-based original indices of every pair, first cap written
  int emit(int32_t* pairs, int64_t cap, int fillzero, int64_t* pairsn);
  // мaxpairs over the current counts (src/gpukernels_cls.jl:109-286)
  int maxpairs(int64_t* out);
  int read_scalar(const int64_t* dev, int64_t* host);
};

}  // namespace gcsph

// opaque C-ABI handle of the cell list (include/gcsph.h)
struct gcl_handle {
  gcsph::CellCore core;
  const double* xuser[3] = {nullptr, nullptr, nullptr};
  gcsph::DevBuf xs[3];
};
