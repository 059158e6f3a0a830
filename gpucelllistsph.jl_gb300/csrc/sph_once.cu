// sph_once.cu -- the pair-once split-row passes of the FP64 step (lanes > 1,
// the default).  Compiled with FMA contraction: these passes are FP64-pipe
// bound on GB300 and contraction removes a multiply or an add from every
// fused product-sum; their results are held to the FP64 contract against the
// oracle (within 1e-12, or the reference's own re-association and rounding
// noise), not bit-identity, which the serial row order in sph_step.cu keeps.
#include "sph_step.cuh"

namespace gcsph {

// fbmolforce!, :1891-1901, for a pair with exactly one real side, at
// separation dx (r2 = |dx|², r = |dx|): adds Δx Fc to f
template <int D>
__device__ inline void fb_pair(const StepConst& c, const double* dx, double r2, double r, double* f) {
  if (dbits(r) < dbits(c.fb_r0)) {
    const double q = c.fb_r0 * rcp_nr(r + c.fb_eta2);
    const double q2 = q * q, q4 = q2 * q2, q8 = q4 * q4, q12 = q8 * q4;
    const double Fc = c.fb_d * (q12 - q4) * rcp_nr(r2 + c.fb_eta2);
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] += dx[d] * Fc;
  }
}

// Pass A: one thread per pair (k, m), k < m in cell order.  Stage 1 at
// (x, ρ, v, P(ρ)) also writes ∇W, and W in the steps that read it; stage 2
// at (xΔt½, ρΔt½, vΔt½, P(ρΔt½)) with the stage-1 ∇W and fbmolforce! at x.
// The reference's terms,
// src/gpukernels_sph.jl, in their algebraically equal pair-once forms:
//  * ∇W = Δx d𝒲/r with d𝒲/r = dWr (1 - u)^3 -- no division by r;
//  * ∂ρ∂tDDT! (:542-631): both sides share DDTkh m₀ (-Δx·∇W)/(r² + η²);
//  * ∂v∂t! (:740-776) and ∂v∂t_av! (:852-901) as one factor of ∇W,
//    -m₀ (Pk + Pm)/(ρk ρm) + 2 α c₀ h m₀ (Δv·Δx)/((r² + η²)(ρk + ρm)).
template <int D, int STAGE>
__device__ __forceinline__ void pairA_one(const StepConst& c, const SArr<D>& S, const PairBuf& B, int64_t u) {
  const int4 q = B.pq[u];
  const int k = q.x, m = q.y, e = q.z;
  int me = q.w;
  if (STAGE == 1 && me < 0) {
    // the partner's row was not staged when the pair list was written: k's
    // position in m's (ascending) row of the finished neighbour list
    int64_t lo = S.rs[m], hi = S.rs[m + 1];
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (S.nbr[mid] < k) lo = mid + 1;
      else hi = mid;
    }
    me = (int)lo;
    B.pq[u] = make_int4(k, m, e, me);
  }
  const double* const* XP = STAGE == 1 ? S.x : S.xh;
  const double* const* VP = STAGE == 1 ? S.v : S.vh;
  const double* RP = STAGE == 1 ? S.rho : S.rhoh;
  const double* PP = STAGE == 1 ? S.P1 : S.P2;
  const double* IP = STAGE == 1 ? S.ir : S.irh;
  double dx[D], dv[D], gw[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dx[d] = XP[d][k] - XP[d][m];
    dv[d] = VP[d][k] - VP[d][m];
  }
  const double r2 = dotD<D>(dx, dx);
  const bool r2pos = dbits(r2) != 0;  // r2 is +0 or positive
  const int ptk = S.pt[k], ptm = S.pt[m];
  const bool mixed = (ptk > 0) != (ptm > 0);
  double r = 0.0;
  if (STAGE == 1) {
    if (r2pos) r = sqrt_nr(r2);
    const double uu = r * c.Hinv;
    double w = 0.0, dwr = 0.0;
    if (dbits(uu) < ONE_BITS) {
      const double t = 1.0 - uu;
      const double t2 = t * t;
      if (c.need_w) w = ((1.0 + 4.0 * uu) * (t2 * t2)) * c.nW;
      dwr = (t2 * t) * c.dWr;
    }
    if (!r2pos) dwr = NAN;  // the reference's d𝒲(0)/0
    if (c.need_w) {
      // both rows' slots: xsphcorr! and cspmcorr! walk every row
      S.We[e] = w;
      S.We[me] = w;
    }
    // stage 2 reads ∇W from the pair's k-side slot only (the call's ∑∇W is
    // recomputed from the positions at its end)
#pragma unroll
    for (int d = 0; d < D; ++d) {
      gw[d] = dx[d] * dwr;
      S.gWe[d][e] = gw[d];
    }
  } else {
    if (c.use_pF && r2pos) r = sqrt_nr(r2);
#pragma unroll
    for (int d = 0; d < D; ++d) gw[d] = S.gWe[d][e];
  }
  const double rk = RP[k], rm = RP[m], irk = IP[k], irm = IP[m];
  const bool both = ptk > 0 && ptm > 0;
  double dk = 0.0, dm = 0.0;
  double sg = ptk * ptm > 0 ? -c.m0 * ((PP[k] + PP[m]) * (irk * irm)) : 0.0;
  double visc = 0.0;
  if (both) {
    const double inv = rcp_nr(r2 + c.eta2);
    const double m0dot = c.m0 * dotD<D>(dv, gw);
    dk = m0dot;
    dm = m0dot;
    if (ptk > 1 || ptm > 1) {
      const double com = c.DDTkhm0 * (-dotD<D>(dx, gw)) * inv;
      const double ez = c.DDTgz * dx[1];
      const double drr = rm - rk;
      if (ptk > 1) {
        const double dp = c.rho0 * (1.0 + pf7m1_fast(ez, c.ginv, c.gamma)) - c.rho0;
        dk += (drr - dp) * com * irm;
      }
      if (ptm > 1) {
        const double dn = c.rho0 * (1.0 + pf7m1_fast(-ez, c.ginv, c.gamma)) - c.rho0;
        dm += (-drr - dn) * com * irk;
      }
    }
    const double cond = dotD<D>(dv, dx);
    const bool av = neg_int(cond);
    if (av || c.use_visc) {
      const double isum = rcp_nr(rk + rm);
      if (av) sg += c.avK * cond * inv * isum;
      if (c.use_visc) visc = 4.0 * c.nu * c.m0 * dotD<D>(dx, gw) * isum * inv;
    }
  }
  double f[D];
#pragma unroll
  for (int d = 0; d < D; ++d) f[d] = c.use_visc ? fma(visc, dv[d], sg * gw[d]) : sg * gw[d];
  if (mixed) {
    if (STAGE == 1) {
      fb_pair<D>(c, dx, r2, r, f);
    } else {
      double dxf[D];
#pragma unroll
      for (int d = 0; d < D; ++d) dxf[d] = S.x[d][k] - S.x[d][m];
      const double r2f = dotD<D>(dxf, dxf);
      fb_pair<D>(c, dxf, r2f, dbits(r2f) != 0 ? sqrt_nr(r2f) : 0.0, f);
    }
  }
  if (c.use_pF) {
    Acc<D> A;
    A.zero();
    pf_term<D>(c, A, ptk, ptm, dx, r);
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] += A.pf[d];
  }
  B.cd[e] = dk;
  B.cd[me] = dm;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    B.ca[d][e] = f[d];
    B.ca[d][me] = -f[d];
  }
}

// Pass A over all pairs in chunks of 32 consecutive pairs, one chunk per warp
// at a time, with one block per SM: PA_TPB threads of about 70 registers
// leave no room for a second block, and the grid is the SM count.  Block b
// takes chunks b, b + G, b + 2G, ... (G blocks) and its warp w every NW-th
// of those, so every SM gets the same number of chunks (to one) -- a grid of
// many small blocks leaves some SMs one block more than others -- and
// consecutive chunks of the cell-ordered list, runs of costly fluid pairs or
// of cheap boundary pairs, go to different SMs.
constexpr int PA_TPB = 768;
template <int D, int STAGE>
__global__ void __launch_bounds__(PA_TPB, 1) k_pairA(StepConst c, SArr<D> S, PairBuf B) {
  if (*S.ovf) return;
  const int64_t np = *B.npair;
  const int64_t G = gridDim.x;
  constexpr int NW = PA_TPB / 32;
  const int lane = threadIdx.x & 31;
  for (int64_t t = threadIdx.x >> 5;; t += NW) {
    const int64_t u0 = ((int64_t)blockIdx.x + G * t) * 32;
    if (u0 >= np) break;
    if (u0 + lane < np) pairA_one<D, STAGE>(c, S, B, u0 + lane);
  }
}

// Pass B: a block of 32 L threads holds 32 particles, L lanes summing each
// row; the sums go through shared memory to warp 0, which runs the
// per-particle update for all 32 at once.  (Run by each group's lane 0, the
// update's divisions and EOS power would issue on the FP64 pipe with 32 / L
// lanes of a warp active: GB300 issues 2 FP64 thread-instructions per cycle
// per SM, so that costs the full warp's time for a few lanes' work.)
template <int D>
struct RowSums {
  double drho[32];
  double a[D][32];
};

template <int D, int L>
__device__ __forceinline__ void pairB_sums(const SArr<D>& S, const PairBuf& B, int64_t N, RowSums<D>& R) {
  const int g = threadIdx.x / L, lane = threadIdx.x % L;
  const int64_t k = (int64_t)blockIdx.x * 32 + g;
  double drho = 0.0, a[D];
#pragma unroll
  for (int d = 0; d < D; ++d) a[d] = 0.0;
  if (k < N) row_sums<D, L>(S, B, k, lane, group_mask<L>(), drho, a);  // whole groups take part
  if (lane == 0) {
    R.drho[g] = drho;
#pragma unroll
    for (int d = 0; d < D; ++d) R.a[d][g] = a[d];
  }
  __syncthreads();
}

// pass B, stage 1: row sums + the three half-step predictors
template <int D, int L>
__global__ void __launch_bounds__(32 * L) k_pairB1(StepConst c, const Scal* __restrict__ sc, int64_t N, SArr<D> S,
                                                   PairBuf B) {
  if (*S.ovf) return;
  __shared__ RowSums<D> R;
  // warp 0 updates the block's 32 particles: their state is loaded before the
  // row sums, so that these loads overlap them (the row sums read only the
  // entry slots)
  const int64_t k = (int64_t)blockIdx.x * 32 + threadIdx.x;
  const bool mine = threadIdx.x < 32 && k < N;
  int ptk = 0;
  double hdt = 0.0, rh0 = 0.0, vh0[D], xh0[D];
  if (mine) {
    ptk = S.pt[k];
    hdt = sc->dt * 0.5;
    rh0 = S.rhoh[k];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      vh0[d] = S.vh[d][k];
      xh0[d] = S.xh[d][k];
    }
  }
  pairB_sums<D, L>(S, B, N, R);
  if (!mine) return;
  double a[D];
#pragma unroll
  for (int d = 0; d < D; ++d) a[d] = R.a[d][threadIdx.x];
  const double drho = R.drho[threadIdx.x];
  a[1] = a[1] - c.g;
  double rv = rh0 + drho * hdt;
  if (rv < c.rho0 && ptk < 0) rv = c.rho0;
  S.rhoh[k] = rv;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double vh = vh0[d];
    if (ptk > 1) vh = vh + a[d] * hdt;
    S.vh[d][k] = vh;
    S.xh[d][k] = xh0[d] + vh * hdt;
  }
  S.P2[k] = eos(rv, c.gamma, c.rho0, c.P0, ptk);
  S.irh[k] = 1.0 / rv;
}

// pass B, stage 2: row sums + symplectic_update! + max |cΔx|; with nb.key
// also the next binning's keys, slots and (last block) cell starts
template <int D, int L>
__global__ void __launch_bounds__(32 * L) k_pairB2(StepConst c, Scal* __restrict__ sc, int64_t N, SArr<D> S,
                                                   PairBuf B, NextBin nb) {
  if (*S.ovf) return;  // uniform over the grid, before the barriers below
  __shared__ RowSums<D> R;
  const bool w0 = threadIdx.x < 32;
  const int64_t k = (int64_t)blockIdx.x * 32 + threadIdx.x;
  // warp 0's particles' state, loaded before the row sums so that these
  // loads overlap them (the row sums read only the entry slots)
  const bool mine = w0 && k < N;
  int ptk = 0;
  double dt = 0.0, p2 = 0.0, rh = 0.0, r0 = 0.0, v0[D], cd0[D], x0[D];
  if (mine) {
    ptk = S.pt[k];
    dt = sc->dt;
    p2 = S.P2[k];
    rh = S.rhoh[k];
    r0 = S.rho[k];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      v0[d] = S.v[d][k];
      cd0[d] = S.cdx[d][k];
      x0[d] = S.x[d][k];
    }
  }
  pairB_sums<D, L>(S, B, N, R);
  if (!w0 && !nb.key) return;
  double mc = 0.0;
  if (mine) {
    double a[D], xn[D];
#pragma unroll
    for (int d = 0; d < D; ++d) a[d] = R.a[d][threadIdx.x];
    const double drho = R.drho[threadIdx.x];
    a[1] = a[1] - c.g;
    S.drho[k] = drho;
    S.Plast[k] = p2;
    const double epsi = -(drho / rh) * dt;
    double rv = r0 * (2.0 - epsi) / (2.0 + epsi);
    if (rv < c.rho0 && ptk <= 1) rv = c.rho0;
    S.rho[k] = rv;
    S.rhoho[k] = rv;
    S.P1[k] = eos(rv, c.gamma, c.rho0, c.P0, ptk);
    S.ir[k] = 1.0 / rv;
    const double ml = ptk > 1 ? 1.0 : 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      S.a[d][k] = a[d];
      const double vv = v0[d];
      const double nv = vv + a[d] * dt * ml;
      S.vho[d][k] = nv;
      S.v[d][k] = nv;
      const double ddx = (vv + nv) * 0.5 * dt;
      const double cd = cd0[d] + ddx;
      S.cdx[d][k] = cd;
      mc = fmax(mc, fabs(cd));
      const double xv = x0[d] + ddx;
      S.xho[d][k] = xv;
      S.xo[d][k] = xv;
      xn[d] = xv;
    }
    if (nb.key) {
      const int32_t ck = cell_key_v<D>(xn, nb.g);
      nb.key[k] = ck;
      nb.slot[k] = atomicAdd(&nb.count[ck], 1);
    }
  }
  if (w0) {
    mc = warp_max(mc);
    __syncwarp();
    if (threadIdx.x == 0) atomic_max_pos(&sc->maxcdx, mc);
  }
  if (nb.key) {
    // the whole block takes part: the last one ends the step (k_step_end's
    // work) and scans the next binning's cell starts, then zeroes the counts
    if (last_block_of_grid(&sc->bdone)) {
      if (threadIdx.x == 0) {
        sc->maxcdx = atomicAdd(&sc->maxcdx, 0ull);  // every block's maximum, seen from here
        step_end_body(c, sc);
      }
      block_exclusive_scan<int32_t>(nb.count, nb.cellstart, nb.g.ncell);
      __syncthreads();
      for (int64_t cc = threadIdx.x; cc < nb.g.ncell; cc += blockDim.x) nb.count[cc] = 0;
    }
    return;
  }
  if (threadIdx.x == 0 && c.fold_end) {
    // the last block to finish ends the step (k_step_end's work); only warp
    // 0 of each block writes step state, and its lane 0 signals here
    __threadfence();
    if (atomicAdd(&sc->bdone, 1u) == gridDim.x - 1) {
      __threadfence();
      sc->maxcdx = atomicAdd(&sc->maxcdx, 0ull);  // every block's maximum, seen from here
      step_end_body(c, sc);
      sc->bdone = 0u;
    }
  }
}


template <int D>
int launch_pairA(int stage, cudaStream_t st, const StepConst& c, const SArr<D>& S, const PairBuf& B) {
  // one block per SM (the kernel's registers and PA_TPB leave room for one);
  // the occupancy query covers a build where two would fit
  static int grid[2] = {0, 0};
  int& g = grid[stage - 1];
  if (g == 0) {
    int dev = 0, sms = 0, per = 0;
    GC_CUDA(cudaGetDevice(&dev));
    GC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (stage == 1)
      GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pairA<D, 1>, PA_TPB, 0));
    else
      GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pairA<D, 2>, PA_TPB, 0));
    g = sms * (per > 0 ? per : 1);
  }
  if (stage == 1)
    k_pairA<D, 1><<<g, PA_TPB, 0, st>>>(c, S, B);
  else
    k_pairA<D, 2><<<g, PA_TPB, 0, st>>>(c, S, B);
  GC_LAUNCHED();
  return GCSPH_OK;
}

template <int D>
int launch_pairB(int stage, int L, int64_t N, cudaStream_t st, const StepConst& c, Scal* sc, const SArr<D>& S,
                 const PairBuf& B, const NextBin* nb) {
  const int g = nblocks(N, 32);  // 32 particles per block, 32 L threads
  NextBin none{};
  const NextBin& nbv = nb ? *nb : none;
#define GC_PAIRB(LL)                                                        \
  if (stage == 1)                                                          \
    k_pairB1<D, LL><<<g, 32 * LL, 0, st>>>(c, sc, N, S, B);                \
  else                                                                     \
    k_pairB2<D, LL><<<g, 32 * LL, 0, st>>>(c, sc, N, S, B, nbv);
  switch (L) {
    case 2: GC_PAIRB(2) break;
    case 4: GC_PAIRB(4) break;
    case 8: GC_PAIRB(8) break;
    case 16: GC_PAIRB(16) break;
    default: GC_PAIRB(32) break;
  }
#undef GC_PAIRB
  GC_LAUNCHED();
  return GCSPH_OK;
}

template int launch_pairA<2>(int, cudaStream_t, const StepConst&, const SArr<2>&, const PairBuf&);
template int launch_pairA<3>(int, cudaStream_t, const StepConst&, const SArr<3>&, const PairBuf&);
template int launch_pairB<2>(int, int, int64_t, cudaStream_t, const StepConst&, Scal*, const SArr<2>&,
                             const PairBuf&, const NextBin*);
template int launch_pairB<3>(int, int, int64_t, cudaStream_t, const StepConst&, Scal*, const SArr<3>&,
                             const PairBuf&, const NextBin*);

}  // namespace gcsph
