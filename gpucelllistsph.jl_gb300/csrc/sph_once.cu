// sph_once.cu -- the pair-once split-row passes of the FP64 step (lanes > 1,
// the default).  Compiled with FMA contraction: these passes are FP64-pipe
// bound on GB300 and contraction removes a multiply or an add from every
// fused product-sum; their results are held to the FP64 contract against the
// oracle (within 1e-12, or the reference's own re-association and rounding
// noise), not bit-identity, which the serial row order in sph_step.cu keeps.
#include "sph_step.cuh"

namespace gcsph {

template <int D, int STAGE>
__global__ void __launch_bounds__(STPB) k_pairA(StepConst c, SArr<D> S, PairBuf B) {
  if (*S.ovf) return;
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= *B.npair) return;
  const int4 q = B.pq[u];
  const int k = q.x, m = q.y, e = q.z, me = q.w;
  // stage 1 at (x, ρ, v, P(ρ)); stage 2 at (xΔt½, ρΔt½, vΔt½, P(ρΔt½)) with stage-1 ∇W, fb at x
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
  double r;
  if (STAGE == 1) {
    const double ri = rsqrt(r2);
    r = r2 > 0.0 ? r2 * ri : 0.0;
    const double u1 = r * c.Hinv;
    const double w = wc2_w(u1, c.nW);
    const double dwk_r = wc2_dw(u1, c.nDW) * ri;
    S.We[e] = w;
    S.We[me] = w;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      gw[d] = dx[d] * dwk_r;
      S.gWe[d][e] = gw[d];
      S.gWe[d][me] = -gw[d];
    }
  } else {
    r = c.use_pF ? (r2 > 0.0 ? r2 * rsqrt(r2) : 0.0) : 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) gw[d] = S.gWe[d][e];
  }
  const int ptk = S.pt[k], ptm = S.pt[m];
  const double rk = RP[k], rm = RP[m], irk = IP[k], irm = IP[m];
  const bool both = ptk > 0 && ptm > 0;
  double dk = 0.0, dm = 0.0;
  const double inv_r2eta = both ? 1.0 / (r2 + c.eta2) : 0.0;
  if (both) {
    // ∂ρ∂tDDT!, src/gpukernels_sph.jl:520-575, both sides of the pair
    const double dot3 = -dotD<D>(dx, gw);
    const double m0dot = c.m0 * dotD<D>(dv, gw);
    dk = m0dot;
    dm = m0dot;
    const double ez = c.DDTgz * dx[1];
    if (ptk > 1) {
      const double dp = c.rho0 * (1.0 + pf7m1_fast(ez, c.ginv, c.gamma)) - c.rho0;
      dk += c.DDTkh * ((rm - rk) - dp) * inv_r2eta * dot3 * c.m0 * irm;
    }
    if (ptm > 1) {
      const double dn = c.rho0 * (1.0 + pf7m1_fast(-ez, c.ginv, c.gamma)) - c.rho0;
      dm += c.DDTkh * ((rk - rm) - dn) * inv_r2eta * dot3 * c.m0 * irk;
    }
  }
  double f[D];
  pair_force_fast<D>(c, ptk, ptm, dx, r2, inv_r2eta, gw, dv, rk, rm, irk, irm, PP[k], PP[m], f);
  double dxf[D];
#pragma unroll
  for (int d = 0; d < D; ++d) dxf[d] = STAGE == 1 ? dx[d] : S.x[d][k] - S.x[d][m];
  pair_tail_terms<D, STAGE>(c, ptk, ptm, dxf, dx, r, f);
  B.cd[e] = dk;
  B.cd[me] = dm;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    B.ca[d][e] = f[d];
    B.ca[d][me] = -f[d];
  }
}

// pass B, stage 1: row sums + the three half-step predictors
template <int D, int L>
__global__ void __launch_bounds__(STPB) k_pairB1(StepConst c, const Scal* __restrict__ sc, int64_t N, SArr<D> S,
                                                 PairBuf B) {
  if (*S.ovf) return;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;  // whole sub-group leaves together
  double drho, a[D];
  row_sums<D, L>(S, B, k, lane, group_mask<L>(), drho, a);
  if (lane != 0) return;
  a[1] = a[1] - c.g;
  const int ptk = S.pt[k];
  const double hdt = sc->dt * 0.5;
  double rv = S.rhoh[k] + drho * hdt;
  if (rv < c.rho0 && ptk < 0) rv = c.rho0;
  S.rhoh[k] = rv;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double vh = S.vh[d][k];
    if (ptk > 1) vh = vh + a[d] * hdt;
    S.vh[d][k] = vh;
    S.xh[d][k] = S.xh[d][k] + vh * hdt;
  }
  S.P2[k] = eos(rv, c.gamma, c.rho0, c.P0, ptk);
  S.irh[k] = 1.0 / rv;
}

// pass B, stage 2: row sums + symplectic_update! + max |cΔx|
template <int D, int L>
__global__ void __launch_bounds__(STPB) k_pairB2(StepConst c, Scal* __restrict__ sc, int64_t N, SArr<D> S,
                                                 PairBuf B) {
  if (*S.ovf) return;  // uniform over the grid, before the block reduction below
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  double mc = 0.0;
  if (k < N) {
    double drho, a[D];
    row_sums<D, L>(S, B, k, lane, group_mask<L>(), drho, a);
    if (lane == 0) {
      const double dt = sc->dt;
      a[1] = a[1] - c.g;
      const int ptk = S.pt[k];
      S.drho[k] = drho;
      S.Plast[k] = S.P2[k];
      const double epsi = -(drho / S.rhoh[k]) * dt;
      double rv = S.rho[k] * (2.0 - epsi) / (2.0 + epsi);
      if (rv < c.rho0 && ptk <= 1) rv = c.rho0;
      S.rho[k] = rv;
      S.rhoho[k] = rv;
      S.P1[k] = eos(rv, c.gamma, c.rho0, c.P0, ptk);
      S.ir[k] = 1.0 / rv;
      const double ml = ptk > 1 ? 1.0 : 0.0;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        S.a[d][k] = a[d];
        const double vv = S.v[d][k];
        const double nv = vv + a[d] * dt * ml;
        S.vho[d][k] = nv;
        S.v[d][k] = nv;
        const double ddx = (vv + nv) * 0.5 * dt;
        const double cd = S.cdx[d][k] + ddx;
        S.cdx[d][k] = cd;
        mc = fmax(mc, fabs(cd));
        const double xv = S.x[d][k] + ddx;
        S.xho[d][k] = xv;
        S.xo[d][k] = xv;
      }
    }
  }
  mc = warp_max(mc);
  __shared__ double smax[STPB / 32];
  if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = smax[0];
    for (int w = 1; w < STPB / 32; ++w) m = fmax(m, smax[w]);
    atomic_max_pos(&sc->maxcdx, m);
    if (c.fold_end) {
      // the last block to finish ends the step (k_step_end's work)
      __threadfence();
      if (atomicAdd(&sc->bdone, 1u) == gridDim.x - 1) {
        __threadfence();
        sc->maxcdx = atomicAdd(&sc->maxcdx, 0ull);  // every block's maximum, seen from here
        step_end_body(c, sc);
        sc->bdone = 0u;
      }
    }
  }
}


template <int D>
int launch_pairA(int stage, int64_t threads, cudaStream_t st, const StepConst& c, const SArr<D>& S,
                 const PairBuf& B) {
  const int g = nblocks(threads, STPB);
  if (stage == 1)
    k_pairA<D, 1><<<g, STPB, 0, st>>>(c, S, B);
  else
    k_pairA<D, 2><<<g, STPB, 0, st>>>(c, S, B);
  GC_LAUNCHED();
  return GCSPH_OK;
}

template <int D>
int launch_pairB(int stage, int L, int64_t N, cudaStream_t st, const StepConst& c, Scal* sc, const SArr<D>& S,
                 const PairBuf& B) {
  const int g = nblocks(N * (int64_t)L, STPB);
#define GC_PAIRB(LL)                                                        \
  if (stage == 1)                                                          \
    k_pairB1<D, LL><<<g, STPB, 0, st>>>(c, sc, N, S, B);                   \
  else                                                                     \
    k_pairB2<D, LL><<<g, STPB, 0, st>>>(c, sc, N, S, B);
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

template int launch_pairA<2>(int, int64_t, cudaStream_t, const StepConst&, const SArr<2>&, const PairBuf&);
template int launch_pairA<3>(int, int64_t, cudaStream_t, const StepConst&, const SArr<3>&, const PairBuf&);
template int launch_pairB<2>(int, int, int64_t, cudaStream_t, const StepConst&, Scal*, const SArr<2>&,
                             const PairBuf&);
template int launch_pairB<3>(int, int, int64_t, cudaStream_t, const StepConst&, Scal*, const SArr<3>&,
                             const PairBuf&);

}  // namespace gcsph
