// sph_step.cu -- SPHProblem + stepsolve! (src/sphproblem.jl:113-345) on sm_103a.
//
// Design: the reference runs ~25-35 one-thread-per-pair kernels per step, each
// scattering FP64 atomics into both particles and each followed by a host
// sync.  Here the particles live in cell order in HBM and every pair pass is a
// GATHER: one thread owns one particle, walks its neighbour CSR (both
// directions, ascending), evaluates each pair term from its own side and
// accumulates in registers.  No atomics, deterministic sums, and the
// per-particle updates are fused into the epilogues:
//   k_stage1 : W, ∇W (stored per CSR entry), ∂ρ∂tDDT!, ∂v∂t!, ∂v∂t_av!,
//              ∂v∂t_visc!, gravity, fbmolforce!(0.4, 2dx), ∂v∂tpF! at (x,ρ,v)
//              + the three half-step predictors + pressure at ρΔt½
//   k_stage2 : the same sums at (xΔt½,ρΔt½,vΔt½) with the stage-1 ∇W,
//              fbmolforce!(bound_D, bound_l) at x + symplectic_update!
//              + pressure at the new ρ + block max of |cΔx|
//   k_dpc, k_xsph, k_cspm : DPC / XSPH / CSPM passes with their updates
// Each term is evaluated from the owning particle's side; the reference's
// j-side formulas are exactly the i-side formula seen from j (negated Δx, Δv
// and ∇W are exact in IEEE arithmetic), so no term changes meaning.
// Arrays that a pass reads from neighbours and also updates are ping-ponged.
#include "sph_step.cuh"

namespace gcsph {
// ---------------------------------------------------------------------------
// stage 1 at (x, ρ, v) + predictors
// ---------------------------------------------------------------------------
template <int D, int L, bool FAST = (L > 1)>
__global__ void __launch_bounds__(STPB) k_stage1(StepConst c, const Scal* __restrict__ sc, int64_t N, SArr<D> S) {
  if (*S.ovf) return;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;  // whole sub-group leaves together
  const unsigned gm = group_mask<L>();
  const double dt = sc->dt;
  double xk[D], vk[D];
#pragma unroll
  for (int d = 0; d < D; ++d) { xk[d] = S.x[d][k]; vk[d] = S.v[d][k]; }
  const double rk = S.rho[k], Pk = S.P1[k];
  const double irk = FAST ? S.ir[k] : 0.0;
  const int ptk = S.pt[k];
  double drho = 0.0;
  Acc<D> A;
  A.zero();
  const int64_t e0 = S.rs[k], e1 = S.rs[k + 1];
  for (int64_t e = e0 + lane; e < e1; e += L) {
    const int32_t m = S.nbr[e];
    double dx[D], dv[D], gw[D];
#pragma unroll
    for (int d = 0; d < D; ++d) { dx[d] = xk[d] - S.x[d][m]; dv[d] = vk[d] - S.v[d][m]; }
    const double r2 = dotD<D>(dx, dx);
    double r, dwk_r;
    if (FAST) {
      const double ri = rsqrt(r2);
      r = r2 > 0.0 ? r2 * ri : 0.0;
      const double u = r * c.Hinv;
      S.We[e] = wc2_w(u, c.nW);
      dwk_r = wc2_dw(u, c.nDW) * ri;
    } else {
      r = sqrt(r2);
      const double u = r * c.Hinv;
      S.We[e] = wc2_w(u, c.nW);                     // sphW!, :84-100
      dwk_r = wc2_dw(u, c.nDW) / r;                 // sph∇W!, :196-213
    }
#pragma unroll
    for (int d = 0; d < D; ++d) { gw[d] = dx[d] * dwk_r; S.gWe[d][e] = gw[d]; }
    const int ptm = S.pt[m];
    const double rm = S.rho[m];
    if (FAST) {
      const bool both = ptk > 0 && ptm > 0;
      const double inv_r2eta = both ? 1.0 / (r2 + c.eta2) : 0.0;
      const double irm = S.ir[m];
      if (both) drho += ddt_term_fast<D>(c, ptk, dx, inv_r2eta, gw, dv, rk, rm, irm);
      mom_terms_fast<D>(c, A, ptk, ptm, dx, inv_r2eta, gw, dv, rk, rm, irk, irm, Pk, S.P1[m]);
    } else {
      if (ptk > 0 && ptm > 0) drho += ddt_term<D>(c, ptk, ptm, dx, r2, gw, dv, rk, rm);
      mom_terms<D>(c, A, ptk, ptm, dx, r2, gw, dv, rk, rm, Pk, S.P1[m]);
    }
    fb_term<D>(c, A, ptk, ptm, dx, r2);
    if (c.use_pF) pf_term<D>(c, A, ptk, ptm, dx, r);
  }
  drho = group_sum<L>(drho, gm);
  group_sum_acc<D, L>(A, c, gm);
  if (lane != 0) return;
  double a[D];
  finish_acc<D>(c, A, a);
  // update_ρp∂ρ∂tΔt!, update_vp∂v∂tΔt!, update_xpvΔt! (:1088-1169), Δt/2
  const double hdt = dt * 0.5;
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
  S.P2[k] = eos(rv, c.gamma, c.rho0, c.P0, ptk);   // pressure! at ρΔt½
  S.irh[k] = 1.0 / rv;
}

// ---------------------------------------------------------------------------
// stage 2 at (xΔt½, ρΔt½, vΔt½) with stage-1 ∇W, + symplectic_update!
// ---------------------------------------------------------------------------
template <int D, int L, bool FAST = (L > 1)>
__global__ void __launch_bounds__(STPB) k_stage2(StepConst c, Scal* __restrict__ sc, int64_t N, SArr<D> S) {
  if (*S.ovf) return;  // uniform over the grid, before the block reduction below
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  double mc = 0.0;
  if (k < N) {
    const unsigned gm = group_mask<L>();
    const double dt = sc->dt;
    double xk[D], xhk[D], vhk[D];
#pragma unroll
    for (int d = 0; d < D; ++d) { xk[d] = S.x[d][k]; xhk[d] = S.xh[d][k]; vhk[d] = S.vh[d][k]; }
    const double rk = S.rhoh[k], Pk = S.P2[k];
    const double irk = FAST ? S.irh[k] : 0.0;
    const int ptk = S.pt[k];
    double drho = 0.0;
    Acc<D> A;
    A.zero();
    const int64_t e0 = S.rs[k], e1 = S.rs[k + 1];
    for (int64_t e = e0 + lane; e < e1; e += L) {
      const int32_t m = S.nbr[e];
      double dx[D], dv[D], gw[D], dxf[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        dx[d] = xhk[d] - S.xh[d][m];
        dv[d] = vhk[d] - S.vh[d][m];
        gw[d] = S.gWe[d][e];
      }
      const double r2 = dotD<D>(dx, dx);
      const int ptm = S.pt[m];
      const double rm = S.rhoh[m];
      if (FAST) {
        const bool both = ptk > 0 && ptm > 0;
        const double inv_r2eta = both ? 1.0 / (r2 + c.eta2) : 0.0;
        const double irm = S.irh[m];
        if (both) drho += ddt_term_fast<D>(c, ptk, dx, inv_r2eta, gw, dv, rk, rm, irm);
        mom_terms_fast<D>(c, A, ptk, ptm, dx, inv_r2eta, gw, dv, rk, rm, irk, irm, Pk, S.P2[m]);
      } else {
        if (ptk > 0 && ptm > 0) drho += ddt_term<D>(c, ptk, ptm, dx, r2, gw, dv, rk, rm);
        mom_terms<D>(c, A, ptk, ptm, dx, r2, gw, dv, rk, rm, Pk, S.P2[m]);
      }
      if ((ptk > 0) != (ptm > 0)) {
#pragma unroll
        for (int d = 0; d < D; ++d) dxf[d] = xk[d] - S.x[d][m];
        fb_term<D>(c, A, ptk, ptm, dxf, dotD<D>(dxf, dxf));
      }
      if (c.use_pF) pf_term<D>(c, A, ptk, ptm, dx, sqrt(r2));
    }
    drho = group_sum<L>(drho, gm);
    group_sum_acc<D, L>(A, c, gm);
    if (lane == 0) {
      double a[D];
      finish_acc<D>(c, A, a);
      S.drho[k] = drho;
      S.Plast[k] = Pk;
      // symplectic_update!, :1204-1245
      const double epsi = -(drho / rk) * dt;
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
        const double xv = xk[d] + ddx;
        S.xho[d][k] = xv;
        S.xo[d][k] = xv;
      }
    }
  }
  // maximum(maximum.(abs, cΔx)), src/sphproblem.jl:325
  mc = warp_max(mc);
  __shared__ double smax[STPB / 32];
  if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = smax[0];
    for (int w = 1; w < STPB / 32; ++w) m = fmax(m, smax[w]);
    atomic_max_pos(&sc->maxcdx, m);
  }
}

// the flat pair list of the pair-once passes: pair u = rs_up[k] + j is k's
// j-th larger-index neighbour m, at entry e of k's row; its mirror is the
// position of k in the smaller-index part of m's row (binary search, the row
// is ascending).  QL lanes per particle share its row tail.
constexpr int QL = 8;
__global__ void __launch_bounds__(256) k_pair_quads(int64_t N, const int64_t* __restrict__ rs,
                                                    const int32_t* __restrict__ nbr,
                                                    const int32_t* __restrict__ cnt_full,
                                                    const int32_t* __restrict__ cnt_up,
                                                    const int64_t* __restrict__ rs_up, const int* __restrict__ ovf,
                                                    int4* __restrict__ pq) {
  if (*ovf) return;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / QL;
  const int lane = (int)(gt % QL);
  if (k >= N) return;
  const int64_t e1 = rs[k + 1];
  const int64_t e0 = e1 - cnt_up[k];
  const int64_t u0 = rs_up[k] - e0;
  for (int64_t e = e0 + lane; e < e1; e += QL) {
    const int32_t m = nbr[e];
    int64_t lo = rs[m], hi = rs[m] + (cnt_full[m] - cnt_up[m]);
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (nbr[mid] < k) lo = mid + 1;
      else hi = mid;
    }
    pq[u0 + e] = make_int4((int)k, (int)m, (int)e, (int)lo);
  }
}

// ---------------------------------------------------------------------------
// dpcreg! + update_dpcreg!  (:1500-1553, :1617-1632)
// ---------------------------------------------------------------------------
template <int D, int L>
__global__ void __launch_bounds__(STPB) k_dpc(StepConst c, const Scal* __restrict__ sc, int64_t N, SArr<D> S) {
  if (*S.ovf) return;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;
  const unsigned gm = group_mask<L>();
  const double dt = sc->dt;
  double xk[D], vk[D], sum[D];
#pragma unroll
  for (int d = 0; d < D; ++d) { xk[d] = S.x[d][k]; vk[d] = S.v[d][k]; sum[d] = 0.0; }
  const double rk = S.rho[k], Pk = S.P1[k];
  const int ptk = S.pt[k];
  const int64_t e0 = S.rs[k], e1 = S.rs[k + 1];
  if (ptk > 0) {
    for (int64_t e = e0 + lane; e < e1; e += L) {
      const int32_t m = S.nbr[e];
      if (!(S.pt[m] > 0)) continue;
      double dx[D], dv[D];
#pragma unroll
      for (int d = 0; d < D; ++d) dx[d] = xk[d] - S.x[d][m];
      const double r2 = dotD<D>(dx, dx);
      // u >= 1: W = 0, so χ = 0, the factor (u >= dpckernlim) is χ and Pᵇ = 0 --
      // the pair adds an exact zero to either branch's sum, which it leaves as
      // it is (up to the sign of a zero sum): skip it.  Past l0² (1 + 1e-6)
      // the rounded u is >= 1 for certain, so most pairs skip before the root
      // (an FP64 square root is some ten FP64-pipe instructions)
      if (r2 > c.dpc_r2cut) continue;
      const double r = sqrt(r2);
      const double u = r * c.dpc_l0inv;
      if (!(u < 1.0)) continue;
#pragma unroll
      for (int d = 0; d < D; ++d) dv[d] = vk[d] - S.v[d][m];
      const double rm = S.rho[m];
      const double w = wc2_w(u, c.dpc_nW);
      const double chi = sqrt(w * c.dpc_whinv);
      const double kk = u < c.dpc_kernlim ? 1.0 : chi;
      const double Pb = chi * jl_max(jl_min(c.dpc_lambda * fabs(Pk + S.P1[m]), c.dpc_lambda * c.dpc_pmax), c.dpc_pmin);
      const double vr = dotD<D>(dv, dx);
      if (vr < 0.0) {
        const double vrdr = vr / (r2 + c.dpc_eta2);
#pragma unroll
        for (int d = 0; d < D; ++d) sum[d] += kk * (-vrdr * dx[d]);
      } else {
        const double tvar = 2.0 * dt * Pb / ((rk + rm) * (r2 + c.dpc_eta2));
#pragma unroll
        for (int d = 0; d < D; ++d) sum[d] += tvar * dx[d];
      }
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) sum[d] = group_sum<L>(sum[d], gm);
  if (lane != 0) return;
  S.Plast[k] = Pk;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    S.buf2[d][k] = sum[d];
    double nv = vk[d], nx = xk[d];
    if (ptk > 1) {
      nv = vk[d] + sum[d];
      nx = xk[d] + sum[d] * dt;
    }
    S.vo[d][k] = nv;
    S.xo[d][k] = nx;
  }
}

// ---------------------------------------------------------------------------
// xsphcorr! + update_xsphcorr!  (:1757-1779, :1827-1838), stage-1 W
// ---------------------------------------------------------------------------
template <int D, int L>
__global__ void __launch_bounds__(STPB) k_xsph(StepConst c, const Scal* __restrict__ sc, int64_t N, SArr<D> S) {
  if (*S.ovf) return;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;
  const unsigned gm = group_mask<L>();
  const double dt = sc->dt;
  double vk[D], sum[D];
#pragma unroll
  for (int d = 0; d < D; ++d) { vk[d] = S.v[d][k]; sum[d] = 0.0; }
  const double rk = S.rho[k];
  const int ptk = S.pt[k];
  if (ptk > 1) {
    const int64_t e0 = S.rs[k], e1 = S.rs[k + 1];
    for (int64_t e = e0 + lane; e < e1; e += L) {
      const int32_t m = S.nbr[e];
      if (!(S.pt[m] > 1)) continue;
      const double xs = c.xsph_c * S.We[e] / (rk + S.rho[m]);
#pragma unroll
      for (int d = 0; d < D; ++d) sum[d] += (S.v[d][m] - vk[d]) * xs;
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) sum[d] = group_sum<L>(sum[d], gm);
  if (lane != 0) return;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    S.buf2[d][k] = sum[d];
    if (ptk > 1) S.x[d][k] = S.x[d][k] + sum[d] * dt;
  }
}

// ---------------------------------------------------------------------------
// cspmcorr!  (:1693-1719), stage-1 W; writes ρ to the other buffer
// ---------------------------------------------------------------------------
template <int D, int L>
__global__ void __launch_bounds__(STPB) k_cspm(StepConst c, int64_t N, SArr<D> S) {
  if (*S.ovf) return;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;
  const unsigned gm = group_mask<L>();
  const double rk = S.rho[k];
  const int ptk = S.pt[k];
  double s1 = 0.0, s2 = 0.0;
  if (ptk > 0) {
    const int64_t e0 = S.rs[k], e1 = S.rs[k + 1];
    for (int64_t e = e0 + lane; e < e1; e += L) {
      const int32_t m = S.nbr[e];
      if (!(S.pt[m] > 0)) continue;
      const double w = S.We[e];
      s1 += c.m0 * w;
      s2 += w * c.m0 / S.rho[m];
    }
  }
  s1 = group_sum<L>(s1, gm);
  s2 = group_sum<L>(s2, gm);
  if (lane != 0) return;
  double nr = s1 / s2;
  double rv = isnan(nr) ? rk : nr;
  S.rhoo[k] = rv;
  S.P1[k] = eos(rv, c.gamma, c.rho0, c.P0, ptk);
  S.ir[k] = 1.0 / rv;
  S.buf2[0][k] = s1;
  S.buf2[1][k] = s2;
  if (D == 3) S.buf2[2][k] = 0.0;
}

// ---------------------------------------------------------------------------
// Δt_stepping (:1293-1353): device maxima, then the scalar update
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(STPB) k_dt_reduce(StepConst c, Scal* __restrict__ sc, int64_t N, SArr<D> S) {
  if (*S.ovf) return;
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double am = 0.0, vm = 0.0;
  if (k < N) {
    double av[D], vv[D], pp[D];
#pragma unroll
    for (int d = 0; d < D; ++d) { av[d] = S.a[d][k]; vv[d] = S.v[d][k]; pp[d] = S.x[d][k]; }
    am = sqrt(dotD<D>(av, av));
    if (!c.dt_relative) {
      // as written at src/gpukernels_sph.jl:1316-1326: absolute positions and velocities
      vm = fabs(c.h * dotD<D>(vv, pp) / (dotD<D>(pp, pp) + c.dt_eta2));
    } else {
      // the viscous time-step bound over pairs: max |h Δv·Δx / (|Δx|² + η²)|
      for (int64_t e = S.rs[k]; e < S.rs[k + 1]; ++e) {
        const int32_t m = S.nbr[e];
        double dx[D], dv[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
          dx[d] = pp[d] - S.x[d][m];
          dv[d] = vv[d] - S.v[d][m];
        }
        vm = fmax(vm, fabs(c.h * dotD<D>(dv, dx) / (dotD<D>(dx, dx) + c.dt_eta2)));
      }
    }
  }
  am = warp_max(am);
  vm = warp_max(vm);
  if ((threadIdx.x & 31) == 0) {
    atomic_max_pos(&sc->amax, am);
    atomic_max_pos(&sc->vmax, vm);
  }
}

__global__ void k_step_end(StepConst c, Scal* __restrict__ sc) {
  if (threadIdx.x != 0 || blockIdx.x != 0 || sc->ovf) return;
  step_end_body(c, sc);
}

// ---------------------------------------------------------------------------
// post-batch sph∑W! + sph∑∇W! (:139-156, :332-359) on original-order arrays
// ---------------------------------------------------------------------------
template <int D, int L>
__global__ void __launch_bounds__(STPB) k_sums_post(StepConst c, int64_t N, const int64_t* __restrict__ rs,
                                                     const int32_t* __restrict__ nbr, const int32_t* __restrict__ orig,
                                                     const int32_t* __restrict__ pt, const double* __restrict__ x0,
                                                     const double* __restrict__ x1, const double* __restrict__ x2,
                                                     double* __restrict__ sumW, double* __restrict__ sg0,
                                                     double* __restrict__ sg1, double* __restrict__ sg2,
                                                     const int* __restrict__ ovf) {
  if (*ovf) return;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = gt / L;
  const int lane = (int)(gt % L);
  if (k >= N) return;
  const unsigned gm = group_mask<L>();
  const double* X[3] = {x0, x1, x2};
  const int32_t o = orig[k];
  double xk[D];
#pragma unroll
  for (int d = 0; d < D; ++d) xk[d] = X[d][o];
  const bool rk = pt[o] > 0;
  double sw = 0.0, sg[D];
#pragma unroll
  for (int d = 0; d < D; ++d) sg[d] = 0.0;
  for (int64_t e = rs[k] + lane; e < rs[k + 1]; e += L) {
    const int32_t om = orig[nbr[e]];
    if ((pt[om] > 0) != rk) continue;
    double dx[D];
#pragma unroll
    for (int d = 0; d < D; ++d) dx[d] = xk[d] - X[d][om];
    const double r = sqrt(dotD<D>(dx, dx));
    const double u = r * c.Hinv;
    sw += wc2_w(u, c.nW);
    const double dwk_r = wc2_dw(u, c.nDW) / r;
#pragma unroll
    for (int d = 0; d < D; ++d) sg[d] += dx[d] * dwk_r;
  }
  sw = group_sum<L>(sw, gm);
#pragma unroll
  for (int d = 0; d < D; ++d) sg[d] = group_sum<L>(sg[d], gm);
  if (lane != 0) return;
  sumW[o] = sw;
  double* SG[3] = {sg0, sg1, sg2};
#pragma unroll
  for (int d = 0; d < D; ++d) SG[d][o] = sg[d];
}

// ---------------------------------------------------------------------------
// state gather (original -> cell order) and scatter (cell -> original order)
// ---------------------------------------------------------------------------
template <int D>
struct StateIO {
  // original-order arrays
  double* x[3];
  double* v[3];
  double* rho;
  const int32_t* pt;
  double* rhoh;
  double* vh[3];
  double* xh[3];
  double* cdx[3];
  double* a[3];
  double* drho;
  double* buf2[3];
  double* P;
};

template <int D>
__global__ void k_gather_state(StepConst c, int64_t N, const int32_t* __restrict__ orig, StateIO<D> O, SArr<D> S) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const int32_t o = orig[k];
  const int pt = O.pt[o];
  ((int32_t*)S.pt)[k] = pt;
  const double r = O.rho[o];
  S.rho[k] = r;
  S.P1[k] = eos(r, c.gamma, c.rho0, c.P0, pt);
  S.ir[k] = 1.0 / r;
  S.rhoh[k] = O.rhoh[o];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    S.x[d][k] = O.x[d][o];
    S.v[d][k] = O.v[d][o];
    S.vh[d][k] = O.vh[d][o];
    S.xh[d][k] = O.xh[d][o];
    S.buf2[d][k] = O.buf2[d][o];
    S.cdx[d][k] = 0.0;  // cΔx reset after update!, src/sphproblem.jl:229
  }
}

// destination buffers of an in-loop re-sort
template <int D>
struct PermOut {
  double* x[3];
  double* xh[3];
  double* v[3];
  double* vh[3];
  double* rho;
  double* rhoh;
  int32_t* pt;
  double* buf2[3];
  // the pair build's FP32 prefilter copy of the new positions and its bound
  // (what the cell list's k_make_pf writes), so that it needs no pass of its own
  float* pf[3];
  unsigned long long* pfmax;
  double off[3];
  float2* thr;     // and its two thresholds, from the last block
  unsigned* cnt;
  double dist2;
};

// the cell-order state of one particle that a re-sort moves
template <int D>
struct PermVals {
  double x[D], xh[D], v[D], vh[D], buf2[D], rho, rhoh;
  int pt;
};
template <int D>
__device__ __forceinline__ PermVals<D> perm_load(const SArr<D>& S, int64_t i) {
  PermVals<D> p;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    p.x[d] = S.x[d][i];
    p.xh[d] = S.xh[d][i];
    p.v[d] = S.v[d][i];
    p.vh[d] = S.vh[d][i];
    p.buf2[d] = S.buf2[d][i];
  }
  p.rho = S.rho[i];
  p.rhoh = S.rhoh[i];
  p.pt = S.pt[i];
  return p;
}
// new[k] = the state p of one particle; cΔx restarts at 0
// (src/sphproblem.jl:229), P(ρ) and 1/ρ are recomputed for stage 1; b takes
// the max |x - offset| of the FP32 prefilter copy
template <int D>
__device__ __forceinline__ void perm_store(const StepConst& c, const SArr<D>& S, const PermOut<D>& O,
                                           const PermVals<D>& p, int64_t k, double& b) {
  double bk = 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    O.x[d][k] = p.x[d];
    const double rel = p.x[d] - O.off[d];
    O.pf[d][k] = (float)rel;
    bk = fmax(bk, fabs(rel));
  }
  if (bk != bk) bk = INFINITY;  // NaN coordinate: every candidate of the set goes to FP64
  b = fmax(b, bk);
  O.pt[k] = p.pt;
  O.rho[k] = p.rho;
  O.rhoh[k] = p.rhoh;
  S.P1[k] = eos(p.rho, c.gamma, c.rho0, c.P0, p.pt);
  S.ir[k] = 1.0 / p.rho;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    O.xh[d][k] = p.xh[d];
    O.v[d][k] = p.v[d];
    O.vh[d][k] = p.vh[d];
    O.buf2[d][k] = p.buf2[d];
    S.cdx[d][k] = 0.0;
  }
}
// new[k] = old[i] for the whole cell-order state of one particle
template <int D>
__device__ __forceinline__ void permute_one(const StepConst& c, const SArr<D>& S, const PermOut<D>& O, int64_t i,
                                            int64_t k, double& b) {
  perm_store<D>(c, S, O, perm_load<D>(S, i), k, b);
}

// new[k] = old[perm[k]] for the whole cell-order state
template <int D>
__global__ void k_permute_state(StepConst c, int64_t N, const int32_t* __restrict__ perm, SArr<D> S, PermOut<D> O) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double b = 0.0;
  if (k < N) permute_one<D>(c, S, O, perm[k], k, b);
  b = warp_max(b);
  if ((threadIdx.x & 31) == 0) atomic_max_pos(O.pfmax, b);
  pf_thresholds_last_block<D>(O.pfmax, O.dist2, O.thr, O.cnt);
}

// The counting sort's rank and the state permute in one pass (sets the
// counting sort orders): the point in arrival position q finds its slot k in
// the new cell order and moves its state there at once -- one launch and one
// read of the map fewer than k_rank_apply followed by k_permute_state.
template <int D>
__global__ void k_rank_permute(StepConst c, int64_t N, const int32_t* __restrict__ tmp,
                               const int32_t* __restrict__ key, const int32_t* __restrict__ cellstart,
                               const int32_t* __restrict__ ord, int32_t* __restrict__ perm,
                               int32_t* __restrict__ skey, int32_t* __restrict__ orig, SArr<D> S, PermOut<D> O,
                               const int32_t* __restrict__ tord) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double b = 0.0;
  if (q < N) {
    // the particle's state is loaded as soon as its index is known, so that
    // these loads overlap the rank's (the rank's stores could alias them)
    const int32_t i = tmp[q];
    const PermVals<D> pv = perm_load<D>(S, i);
    const int64_t k = rank_in_cell(tmp, key, cellstart, ord, q, perm, skey, orig, nullptr, tord);
    perm_store<D>(c, S, O, pv, k, b);
  }
  b = warp_max(b);
  if ((threadIdx.x & 31) == 0) atomic_max_pos(O.pfmax, b);
  pf_thresholds_last_block<D>(O.pfmax, O.dist2, O.thr, O.cnt);
}

template <int D>
__global__ void k_scatter_state(int64_t N, const int32_t* __restrict__ orig, StateIO<D> O, SArr<D> S) {
  if (*S.ovf) return;  // a captured call that overflowed leaves the caller's arrays untouched
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const int32_t o = orig[k];
  O.rho[o] = S.rho[k];
  O.rhoh[o] = S.rhoh[k];
  O.drho[o] = S.drho[k];
  O.P[o] = S.Plast[k];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    O.x[d][o] = S.x[d][k];
    O.v[d][o] = S.v[d][k];
    O.vh[d][o] = S.vh[d][k];
    O.xh[d][o] = S.xh[d][k];
    O.cdx[d][o] = S.cdx[d][k];
    O.a[d][o] = S.a[d][k];
    O.buf2[d][o] = S.buf2[d][k];
  }
}

}  // namespace gcsph

// ===========================================================================
// host side
// ===========================================================================
using namespace gcsph;

// captured stepsolve! calls (see step_graph)
struct HostSide {
  int idx[6];
  void* pt[2];
  void* buf2[3][2];
  void* orig[2];
  bool sorted, built, up_valid, in_cell_order, rows_upper;
  int64_t nfull;
};

struct GraphKey {
  int32_t n, timestepping, lanes, timing, dt_relative, pad;
  double tmin, tmax;
  gcsph_params prm;  // dt and etime zeroed: they live on the device
  int64_t nbr_cap, we_cap, gen;
  HostSide at;       // buffer indices and pointer pairs at the start
  const void* user[8];  // the caller's arrays the call reads and writes
};

struct StepGraph {
  GraphKey key;
  cudaGraphExec_t exec = nullptr;
  HostSide after{};
  long long launches = 0;
  std::vector<TimerRec> timers;
  unsigned long long used = 0;
};

static void graph_free(StepGraph& g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  g.exec = nullptr;
  timer_release(g.timers);
}

struct sph_handle {
  gcl_handle* cl = nullptr;
  int D = 2;
  int64_t N = 0;
  gcsph_params prm{};
  // caller arrays (original order)
  double* rho_u = nullptr;
  double* v_u[3] = {nullptr, nullptr, nullptr};
  const int32_t* pt_u = nullptr;
  DevBuf vown[3];
  // library-owned original-order arrays
  DevBuf rhoh_o, vh_o[3], xh_o[3], cdx_o[3], P_o, a_o[3], drho_o, buf2_o[3], sumW_o, sumgW_o[3];
  // cell-order working arrays
  DevBuf X[2][3], XH[2][3], V[2][3], VH[2][3], RHO[2], RHOH[2], P1, P2, PT, A[3], DRHO, CDX[3], BUF2[3], PLAST, We,
      GWe[3], IR, IRH;
  DevBuf PT_b, BUF2_b[3];  // spares for the in-loop re-sort
  DevBuf CD, CA[3], PQ;     // pair-once passes: per-entry contributions, flat pair list
  int ix = 0, ixh = 0, iv = 0, ivh = 0, irho = 0, irhoh = 0;
  int64_t we_cap = 0;
  int lanes = 0;  // lanes per particle in the pair passes; 0 = by mean row length
  DevBuf scal;
  Scal* pin = nullptr;
  bool in_cell_order = false;
  bool keys_ready = false;  // pass B2 wrote the next binning's keys (captured calls)
  bool use_graphs = true;
  int dt_relative = 0;
  StepGraph graphs[4];
  unsigned long long graph_clock = 0;
  int64_t n_captures = 0, n_replays = 0;
  cudaStream_t cap_stream = nullptr;  // records captures only; replays run on the cell list's stream
};

static StepConst make_const(const sph_handle* h) {
  const gcsph_params& p = h->prm;
  StepConst c{};
  c.h = p.h;
  c.eta2 = (0.1 * p.h) * (0.1 * p.h);
  c.m0 = p.m0;
  c.rho0 = p.rho0;
  c.gamma = p.gamma;
  c.ginv = 1.0 / (double)p.gamma;
  c.DDTkh = 2.0 * p.h * p.delta * p.c0;
  double Cb = (p.c0 * p.c0 * p.rho0) * c.ginv;
  c.DDTgz = p.rho0 * p.g / Cb;
  c.P0 = p.c0 * p.c0 * p.rho0 / (double)p.gamma;
  c.alpha = p.alpha;
  c.c0 = p.c0;
  c.nu = p.nu;
  c.g = p.g;
  c.s = p.s;
  c.Hinv = 1.0 / p.H;
  if (h->D == 2) {
    c.nW = wc2_norm_w<2>(c.Hinv);
    c.nDW = wc2_norm_dw<2>(c.Hinv);
  } else {
    c.nW = wc2_norm_w<3>(c.Hinv);
    c.nDW = wc2_norm_dw<3>(c.Hinv);
  }
  c.dWr = -20.0 * c.nDW * c.Hinv;
  c.DDTkhm0 = c.DDTkh * p.m0;
  c.avK = 2.0 * p.alpha * p.c0 * p.h * p.m0;
  c.twoh = 2.0 * p.h;
  c.pfc = 1.5 * GCSPH_PI64;
  c.hp1 = 0.1 * p.h;
  c.use_visc = p.nu > 0;
  c.use_pF = p.s > 0;
  if (p.dpc_l0 > 0) {
    c.dpc_l0inv = 1.0 / p.dpc_l0;
    c.dpc_r2cut = p.dpc_l0 * p.dpc_l0 * (1.0 + 1e-6);
    c.dpc_nW = h->D == 2 ? wc2_norm_w<2>(c.dpc_l0inv) : wc2_norm_w<3>(c.dpc_l0inv);
    c.dpc_whinv = 1.0 / wc2_w(0.5, c.dpc_nW);
    c.dpc_pmin = p.dpc_pmin;
    c.dpc_pmax = p.dpc_pmax;
    c.dpc_lambda = p.dpc_lambda;
    c.dpc_kernlim = gcsph_dpckernlim(h->D);
    c.dpc_eta2 = (0.1 * p.dpc_l0) * (0.1 * p.dpc_l0);
  }
  c.xsph_c = 2.0 * p.m0 * p.xsph_eps;
  c.cfl = p.CFL;
  c.dt_eta2 = (0.01 * p.h) * (0.01 * p.h);
  return c;
}

template <int D>
static SArr<D> make_arr(sph_handle* h) {
  SArr<D> S{};
  CellCore& core = h->cl->core;
  S.rs = core.rs_full.as<int64_t>();
  S.nbr = core.nbr.as<int32_t>();
  S.pt = h->PT.as<int32_t>();
  S.orig = core.orig.as<int32_t>();
  for (int d = 0; d < D; ++d) {
    S.x[d] = h->X[h->ix][d].as<double>();
    S.xo[d] = h->X[h->ix ^ 1][d].as<double>();
    S.v[d] = h->V[h->iv][d].as<double>();
    S.vo[d] = h->V[h->iv ^ 1][d].as<double>();
    S.xh[d] = h->XH[h->ixh][d].as<double>();
    S.xho[d] = h->XH[h->ixh ^ 1][d].as<double>();
    S.vh[d] = h->VH[h->ivh][d].as<double>();
    S.vho[d] = h->VH[h->ivh ^ 1][d].as<double>();
    S.gWe[d] = h->GWe[d].as<double>();
    S.a[d] = h->A[d].as<double>();
    S.cdx[d] = h->CDX[d].as<double>();
    S.buf2[d] = h->BUF2[d].as<double>();
  }
  S.rho = h->RHO[h->irho].as<double>();
  S.rhoo = h->RHO[h->irho ^ 1].as<double>();
  S.rhoh = h->RHOH[h->irhoh].as<double>();
  S.rhoho = h->RHOH[h->irhoh ^ 1].as<double>();
  S.P1 = h->P1.as<double>();
  S.P2 = h->P2.as<double>();
  S.ir = h->IR.as<double>();
  S.irh = h->IRH.as<double>();
  S.We = h->We.as<double>();
  S.drho = h->DRHO.as<double>();
  S.Plast = h->PLAST.as<double>();
  S.ovf = &h->scal.as<Scal>()->ovf;
  return S;
}

template <int D>
static PermOut<D> make_alt(sph_handle* h) {
  PermOut<D> O{};
  for (int d = 0; d < D; ++d) {
    O.x[d] = h->X[h->ix ^ 1][d].as<double>();
    O.xh[d] = h->XH[h->ixh ^ 1][d].as<double>();
    O.v[d] = h->V[h->iv ^ 1][d].as<double>();
    O.vh[d] = h->VH[h->ivh ^ 1][d].as<double>();
    O.buf2[d] = h->BUF2_b[d].as<double>();
  }
  O.rho = h->RHO[h->irho ^ 1].as<double>();
  O.rhoh = h->RHOH[h->irhoh ^ 1].as<double>();
  O.pt = h->PT_b.as<int32_t>();
  return O;
}

// W and ∇W per neighbour entry follow the neighbour CSR's capacity
template <int D>
static int grow_entry_arrays(sph_handle* h) {
  CellCore& core = h->cl->core;
  if (core.nbr_cap <= h->we_cap) return GCSPH_OK;
  const int64_t want = core.nbr_cap;
  int rc;
  if ((rc = h->We.ensure(sizeof(double) * want, core.st))) return rc;
  if ((rc = h->CD.ensure(sizeof(double) * want, core.st))) return rc;
  if (want / 2 + 1 > (int64_t)INT32_MAX) return fail(GCSPH_ECAPACITY, "neighbour entries past 2^31");
  if ((rc = h->PQ.ensure(sizeof(int4) * (want / 2 + 1), core.st))) return rc;
  for (int d = 0; d < D; ++d) {
    if ((rc = h->GWe[d].ensure(sizeof(double) * want, core.st))) return rc;
    if ((rc = h->CA[d].ensure(sizeof(double) * want, core.st))) return rc;
  }
  h->we_cap = want;
  return GCSPH_OK;
}

template <int D>
static PairBuf make_pairbuf(sph_handle* h) {
  PairBuf B{};
  B.cd = h->CD.as<double>();
  for (int d = 0; d < D; ++d) B.ca[d] = h->CA[d].as<double>();
  B.pq = h->PQ.as<int4>();
  B.npair = h->cl->core.rs_up.as<int64_t>() + h->N;
  return B;
}

template <int D>
static StateIO<D> make_io(sph_handle* h) {
  StateIO<D> O{};
  for (int d = 0; d < D; ++d) {
    O.x[d] = (double*)h->cl->xuser[d];
    O.v[d] = h->v_u[d];
    O.vh[d] = h->vh_o[d].as<double>();
    O.xh[d] = h->xh_o[d].as<double>();
    O.cdx[d] = h->cdx_o[d].as<double>();
    O.a[d] = h->a_o[d].as<double>();
    O.buf2[d] = h->buf2_o[d].as<double>();
  }
  O.rho = h->rho_u;
  O.pt = h->pt_u;
  O.rhoh = h->rhoh_o.as<double>();
  O.drho = h->drho_o.as<double>();
  O.P = h->P_o.as<double>();
  return O;
}

template <int D>
static int scatter_state(sph_handle* h) {
  CellCore& core = h->cl->core;
  timer_begin(T_STATE, core.st);
  k_scatter_state<D><<<nblocks(h->N, 256), 256, 0, core.st>>>(h->N, core.orig.as<int32_t>(), make_io<D>(h),
                                                             make_arr<D>(h));
  GC_LAUNCHED();
  timer_end(T_STATE, core.st);
  h->in_cell_order = false;
  return GCSPH_OK;
}

// update! inside stepsolve!: bin the original-order points, sort, gather the
// whole state into cell order, rebuild the neighbour CSR
template <int D>
static int rebuild(sph_handle* h, const StepConst& c, int* ovf_dev) {
  CellCore& core = h->cl->core;
  int rc;
  bool pf_ready = false;
  if (!h->in_cell_order) {
    // first update! of a call: bin the original-order points and gather the state
    if ((rc = core.sort(h->cl->xuser, nullptr))) return rc;
    h->ix = h->ixh = h->iv = h->ivh = h->irho = h->irhoh = 0;
    timer_begin(T_STATE, core.st);
    k_gather_state<D><<<nblocks(h->N, 256), 256, 0, core.st>>>(c, h->N, core.orig.as<int32_t>(), make_io<D>(h),
                                                              make_arr<D>(h));
    GC_LAUNCHED();
    timer_end(T_STATE, core.st);
    h->in_cell_order = true;
  } else {
    // update! inside the loop: re-bin the cell-ordered points, ties broken by
    // original index (the same canonical order), then permute the state from
    // the old cell order straight into the new one
    const double* xc[3] = {h->X[h->ix][0].as<double>(), h->X[h->ix][1].as<double>(),
                           D == 3 ? h->X[h->ix][2].as<double>() : nullptr};
    bool rank_deferred = false;
    const bool keys_ready = h->keys_ready;
    h->keys_ready = false;
    if ((rc = core.sort(xc, core.orig.as<int32_t>(), false, &rank_deferred, keys_ready))) return rc;
    if ((rc = core.ensure_pf())) return rc;
    PermOut<D> alt = make_alt<D>(h);
    for (int d = 0; d < D; ++d) {
      alt.pf[d] = core.pf[d].as<float>();
      alt.off[d] = core.g.offset[d];
    }
    alt.pfmax = core.pfmax.as<unsigned long long>();
    alt.thr = core.pfthr.as<float2>();
    alt.cnt = core.pfcnt.as<unsigned>();
    alt.dist2 = core.g.dist2;
    // small sets: 64-thread blocks, so the latency-bound passes spread over more SMs
    const int ptb = h->N <= RADIX_MIN_N ? 64 : 256;
    if (rank_deferred) {
      timer_begin(T_STATE, core.st);
      k_rank_permute<D><<<nblocks(h->N, ptb), ptb, 0, core.st>>>(
          c, h->N, core.tmp.as<int32_t>(), core.key.as<int32_t>(), core.cellstart.as<int32_t>(),
          core.orig.as<int32_t>(), core.perm.as<int32_t>(), core.skey.as<int32_t>(), core.orig_b.as<int32_t>(),
          make_arr<D>(h), alt, core.tord.as<int32_t>());
      GC_LAUNCHED();
      timer_end(T_STATE, core.st);
      core.sort_done();
    } else {
      timer_begin(T_STATE, core.st);
      k_permute_state<D><<<nblocks(h->N, ptb), ptb, 0, core.st>>>(c, h->N, core.perm.as<int32_t>(), make_arr<D>(h),
                                                                 alt);
      GC_LAUNCHED();
      timer_end(T_STATE, core.st);
    }
    pf_ready = true;
    h->ix ^= 1;
    h->ixh ^= 1;
    h->iv ^= 1;
    h->ivh ^= 1;
    h->irho ^= 1;
    h->irhoh ^= 1;
    std::swap(h->PT.p, h->PT_b.p);
    std::swap(h->PT.bytes, h->PT_b.bytes);
    for (int d = 0; d < D; ++d) {
      std::swap(h->BUF2[d].p, h->BUF2_b[d].p);
      std::swap(h->BUF2[d].bytes, h->BUF2_b[d].bytes);
    }
  }
  const double* xs[3] = {h->X[h->ix][0].as<double>(), h->X[h->ix][1].as<double>(),
                         D == 3 ? h->X[h->ix][2].as<double>() : nullptr};
  // the flat pair list comes with the fill when the capacity stays (pass A
  // resolves the mirror of a pair whose partner's row was too long to stage)
  bool pq_done = false;
  int4* pq = h->we_cap >= core.nbr_cap && core.nbr_cap > 0 ? h->PQ.as<int4>() : nullptr;
  if ((rc = core.build_pairs(xs, ovf_dev, true, pf_ready, pq, &pq_done))) return rc;
  if ((rc = grow_entry_arrays<D>(h))) return rc;
  if (!pq_done) {
    // flat pair list: offsets scanned with the row offsets (no read-back), then the quads
    timer_begin(T_PAIRS, core.st);
    k_pair_quads<<<nblocks(h->N * QL, 256), 256, 0, core.st>>>(
        h->N, core.rs_full.as<int64_t>(), core.nbr.as<int32_t>(), core.cnt_full.as<int32_t>(),
        core.cnt_up.as<int32_t>(), core.rs_up.as<int64_t>(), ovf_dev, h->PQ.as<int4>());
    GC_LAUNCHED();
    timer_end(T_PAIRS, core.st);
  }
  return GCSPH_OK;
}

// L lanes per particle: one launch per pair pass, N*L threads
#define PAIR_LAUNCH(KER, L, ...)                                                              \
  do {                                                                                        \
    const int _g = nblocks(h->N * (int64_t)(L), STPB);                                        \
    switch (L) {                                                                              \
      case 1: KER<D, 1><<<_g, STPB, 0, st>>>(__VA_ARGS__); break;                             \
      case 2: KER<D, 2><<<_g, STPB, 0, st>>>(__VA_ARGS__); break;                             \
      case 4: KER<D, 4><<<_g, STPB, 0, st>>>(__VA_ARGS__); break;                             \
      case 8: KER<D, 8><<<_g, STPB, 0, st>>>(__VA_ARGS__); break;                             \
      case 16: KER<D, 16><<<_g, STPB, 0, st>>>(__VA_ARGS__); break;                           \
      default: KER<D, 32><<<_g, STPB, 0, st>>>(__VA_ARGS__); break;                           \
    }                                                                                         \
  } while (0)

// pass A: one thread per pair, one block per SM (the pair count itself
// stays on the device); pass B: L lanes per row
#define PAIRA_LAUNCH(STAGE, ...)                                                              \
  do {                                                                                        \
    const int _rc = launch_pairA<D>(STAGE, st, __VA_ARGS__);                                  \
    if (_rc) return _rc;                                                                      \
  } while (0)

#define PAIRB_LAUNCH(STAGE, L, ...)                                                           \
  do {                                                                                        \
    const int _rc = launch_pairB<D>(STAGE, L, h->N, st, __VA_ARGS__);                        \
    if (_rc) return _rc;                                                                      \
  } while (0)

static int choose_lanes(const sph_handle* h) {
  if (h->lanes > 0) return h->lanes;
  const CellCore& core = h->cl->core;
  double mean = h->N > 0 ? (double)core.nfull_est / (double)h->N : 0.0;
  // about four neighbours per lane
  int L = 1;
  while (L < 32 && (double)L * 4.0 < mean) L <<= 1;
  return L;
}

template <int D>
static int finish_call(sph_handle* h, const StepConst& c, Scal* dsc) {
  CellCore& core = h->cl->core;
  cudaStream_t st = core.st;
  int rc;
  if (h->in_cell_order && (rc = scatter_state<D>(h))) return rc;
  if (core.built && core.rows_upper) {
    // no update! ran in this call (n = 0) and the last pair set is the cell
    // list's own update!, which stores the larger-index half of each row:
    // the same set again with full rows, on the points it was binned from
    const double* xs[3] = {h->cl->xs[0].as<double>(), h->cl->xs[1].as<double>(),
                           D == 3 ? h->cl->xs[2].as<double>() : nullptr};
    if ((rc = core.build_pairs(xs, nullptr, true))) return rc;
  }
  // post-batch ∑W, ∑∇W on the last pair set and the final points
  if (core.built) {
    const double* x2 = D == 3 ? h->cl->xuser[2] : h->cl->xuser[0];
    double* sg2 = D == 3 ? h->sumgW_o[2].as<double>() : h->sumgW_o[0].as<double>();
    timer_begin(T_POST, st);
    const int L = choose_lanes(h);
    PAIR_LAUNCH(k_sums_post, L, c, h->N, core.rs_full.as<int64_t>(), core.nbr.as<int32_t>(),
                                        core.orig.as<int32_t>(), h->pt_u, h->cl->xuser[0], h->cl->xuser[1], x2,
                                        h->sumW_o.as<double>(), h->sumgW_o[0].as<double>(),
                                        h->sumgW_o[1].as<double>(), sg2, &dsc->ovf);
    GC_LAUNCHED();
    timer_end(T_POST, st);
  }
  return GCSPH_OK;
}

// everything of one step after update!: both stages, DPC, XSPH, CSPM, Δt.
// Shared by the eager loop and the graph capture; only the host-side buffer
// indices change here, in an order fixed by the parameters.
template <int D>
// next_bins: update! starts the next step (captured calls): pass B2 may
// start its binning (NextBin)
static int enqueue_stages(sph_handle* h, StepConst& c, Scal* dsc, int32_t& cspmcnt, bool next_bins) {
  CellCore& core = h->cl->core;
  cudaStream_t st = core.st;
  const gcsph_params& p = h->prm;
  const int nb = nblocks(h->N, STPB);
  cspmcnt += 1;
  c.fb_d = 0.4;
  c.fb_r0 = 2.0 * p.dx;
  c.fb_eta2 = 0.01 * (c.fb_r0 * c.fb_r0);
  const int L = choose_lanes(h);
  const bool once = L > 1;  // pair-once passes; L = 1 keeps the serial gather (bit-identical to the oracle)
  // W of the pairs is read by xsphcorr! and by a CSPM step's cspmcorr! only
  // (the call's ∑W is recomputed from the positions at its end)
  c.need_w = (p.xsph_eps > 0) || (p.cspmn > 0 && cspmcnt == p.cspmn);
  bool folded = false;  // k_step_end's work done by pass B2's last block
  // stage 1 (predictor) and stage 2 (corrector); the pair-once form times
  // pass A as the stage and the two row-sum passes together
  if (once) {
    timer_begin(T_STAGE1, st);
    PAIRA_LAUNCH(1, c, make_arr<D>(h), make_pairbuf<D>(h));
    timer_end(T_STAGE1, st);
    timer_begin(T_ROWSUM, st);
    PAIRB_LAUNCH(1, L, c, dsc, make_arr<D>(h), make_pairbuf<D>(h));
    timer_end(T_ROWSUM, st);
  } else {
    timer_begin(T_STAGE1, st);
    PAIR_LAUNCH(k_stage1, L, c, dsc, h->N, make_arr<D>(h));
    GC_LAUNCHED();
    timer_end(T_STAGE1, st);
  }
  c.fb_d = p.bound_D;
  c.fb_r0 = p.bound_l;
  c.fb_eta2 = 0.01 * (c.fb_r0 * c.fb_r0);
  if (once) {
    timer_begin(T_STAGE2, st);
    PAIRA_LAUNCH(2, c, make_arr<D>(h), make_pairbuf<D>(h));
    timer_end(T_STAGE2, st);
    timer_begin(T_ROWSUM, st);
    // without Δt_stepping nothing after pass B2 feeds the step's end: its
    // last block does k_step_end's work
    StepConst c2 = c;
    c2.fold_end = c.timestepping ? 0 : 1;
    // the next binning's keys from the new positions, where nothing after
    // pass B2 moves the particles (no DPC, no XSPH) and its last block ends the step
    NextBin nb{};
    if (next_bins && c2.fold_end && !(p.dpc_l0 > 0) && !(p.xsph_eps > 0) && core.keys_in_step()) {
      nb.key = core.key.as<int32_t>();
      nb.slot = core.slot.as<int32_t>();
      nb.count = core.count.as<int32_t>();
      nb.cellstart = core.cellstart.as<int32_t>();
      nb.g = core.g;
      h->keys_ready = true;
    }
    PAIRB_LAUNCH(2, L, c2, dsc, make_arr<D>(h), make_pairbuf<D>(h), &nb);
    folded = c2.fold_end != 0;
    timer_end(T_ROWSUM, st);
  } else {
    timer_begin(T_STAGE2, st);
    PAIR_LAUNCH(k_stage2, L, c, dsc, h->N, make_arr<D>(h));
    GC_LAUNCHED();
    timer_end(T_STAGE2, st);
  }
  h->ix ^= 1;
  h->ixh ^= 1;
  h->ivh ^= 1;
  h->irhoh ^= 1;
  if (p.dpc_l0 > 0) {
    timer_begin(T_DPC, st);
    PAIR_LAUNCH(k_dpc, L, c, dsc, h->N, make_arr<D>(h));
    GC_LAUNCHED();
    timer_end(T_DPC, st);
    h->iv ^= 1;
    h->ix ^= 1;
  }
  if (p.xsph_eps > 0) {
    timer_begin(T_XSPH, st);
    PAIR_LAUNCH(k_xsph, L, c, dsc, h->N, make_arr<D>(h));
    GC_LAUNCHED();
    timer_end(T_XSPH, st);
  }
  if (p.cspmn > 0 && cspmcnt == p.cspmn) {
    timer_begin(T_CSPM, st);
    PAIR_LAUNCH(k_cspm, L, c, h->N, make_arr<D>(h));
    GC_LAUNCHED();
    timer_end(T_CSPM, st);
    h->irho ^= 1;
    cspmcnt = 0;
  }
  if (c.timestepping) {
    timer_begin(T_DT, st);
    k_dt_reduce<D><<<nb, STPB, 0, st>>>(c, dsc, h->N, make_arr<D>(h));
    GC_LAUNCHED();
    timer_end(T_DT, st);
  }
  if (!folded) {
    k_step_end<<<1, 32, 0, st>>>(c, dsc);
    GC_LAUNCHED();
  }
  return GCSPH_OK;
}

// device scalars at the start of a call
static void init_scal(sph_handle* h, int32_t n) {
  h->pin->dt = h->prm.dt;
  h->pin->etime = h->prm.etime;
  h->pin->maxcdx = h->pin->amax = h->pin->vmax = 0;
  h->pin->ovf = 0;
  h->pin->bdone = 0;
  h->pin->maxout = 0;
  h->pin->nreb = n > 0 ? 1 : 0;  // the first step always runs update!
}

// _stepsolve!, one host round trip per step: the host reads the step's
// scalars, decides update!, and on a neighbour overflow grows and repeats
template <int D>
static int step_eager(sph_handle* h, StepConst c, int32_t n, int64_t* updaten_out, double* maxcdx_out) {
  CellCore& core = h->cl->core;
  cudaStream_t st = core.st;
  Scal* dsc = h->scal.as<Scal>();
  init_scal(h, n);
  GC_CUDA(cudaMemcpyAsync(dsc, h->pin, sizeof(Scal), cudaMemcpyHostToDevice, st));
  bool skip = false;
  int64_t updaten = 0;
  double maxout = 0.0;
  int32_t cspmcnt = 0;
  int rc;
  c.count_reb = 0;
  h->keys_ready = false;  // the eager loop bins every step itself
  for (int32_t it = 0; it < n; ++it) {
    const int32_t cspm_before = cspmcnt;
    // per-step device scalars: max|cΔx|, the Δt maxima and the overflow flag
    GC_CUDA(cudaMemsetAsync(&dsc->maxcdx, 0, 4 * sizeof(unsigned long long), st));
    if (!skip) {
      if ((rc = rebuild<D>(h, c, &dsc->ovf))) return rc;
      skip = true;
      updaten += 1;
    }
    const int saved[6] = {h->ix, h->ixh, h->iv, h->ivh, h->irho, h->irhoh};
    if ((rc = enqueue_stages<D>(h, c, dsc, cspmcnt, false))) return rc;
    GC_CUDA(cudaMemcpyAsync(h->pin, dsc, sizeof(Scal), cudaMemcpyDeviceToHost, st));
    GC_CUDA(cudaStreamSynchronize(st));
    timer_collect();
    if (h->pin->ovf) {
      // the rebuilt neighbour CSR did not fit: every kernel of this step
      // skipped, so the state is the re-sorted one -- grow and repeat the step
      h->ix = saved[0];
      h->ixh = saved[1];
      h->iv = saved[2];
      h->ivh = saved[3];
      h->irho = saved[4];
      h->irhoh = saved[5];
      if ((rc = core.read_nfull())) return rc;
      if ((rc = core.grow_nbr(core.nfull))) return rc;
      if ((rc = grow_entry_arrays<D>(h))) return rc;
      cspmcnt = cspm_before;
      skip = false;
      updaten -= 1;
      it -= 1;
      continue;
    }
    unsigned long long bits = h->pin->maxcdx;
    double mc;
    memcpy(&mc, &bits, 8);
    if (mc > c.reb_thr) skip = false;
    if (mc > maxout) maxout = mc;
  }
  if ((rc = finish_call<D>(h, c, dsc))) return rc;
  GC_CUDA(cudaMemcpyAsync(h->pin, dsc, sizeof(Scal), cudaMemcpyDeviceToHost, st));
  GC_CUDA(cudaStreamSynchronize(st));
  timer_collect();
  h->prm.dt = h->pin->dt;
  h->prm.etime = h->pin->etime;
  if (updaten_out) *updaten_out = updaten;
  if (maxcdx_out) *maxcdx_out = maxout;
  return GCSPH_OK;
}

// ---------------------------------------------------------------------------
// Captured calls.  When update! is due after every step (nui <= 0, as with
// dist = H), a whole stepsolve! call -- gather, n x (update!, stages, Δt),
// scatter, post sums -- is one CUDA graph, replayed with one host round trip.
// The decisions the eager loop takes on the host move to the device:
// k_step_end counts update! calls and keeps the largest max|cΔx| the way the
// host loop does.  update! also runs after a step whose max|cΔx| is exactly
// 0 (nothing moved), where the host loop skips it: the re-sort of unmoved
// points by (cell, original index) is the identity and the pair set is the
// same, so the state is too.  A neighbour overflow inside the replay skips
// every later kernel, the final scatter included, so the caller's
// original-order arrays still hold the call's inputs: the host grows the
// buffers and runs the call again eagerly.
// ---------------------------------------------------------------------------
static HostSide host_side(const sph_handle* h) {
  HostSide s{};
  const CellCore& core = h->cl->core;
  s.idx[0] = h->ix;
  s.idx[1] = h->ixh;
  s.idx[2] = h->iv;
  s.idx[3] = h->ivh;
  s.idx[4] = h->irho;
  s.idx[5] = h->irhoh;
  s.pt[0] = h->PT.p;
  s.pt[1] = h->PT_b.p;
  for (int d = 0; d < 3; ++d) {
    s.buf2[d][0] = h->BUF2[d].p;
    s.buf2[d][1] = h->BUF2_b[d].p;
  }
  s.orig[0] = core.orig.p;
  s.orig[1] = core.orig_b.p;
  s.sorted = core.sorted;
  s.built = core.built;
  s.up_valid = core.up_valid;
  s.rows_upper = core.rows_upper;
  s.in_cell_order = h->in_cell_order;
  s.nfull = core.nfull;
  return s;
}

// the pairs swapped by the re-sorts are equal-sized, so pointers alone move
static void set_host_side(sph_handle* h, const HostSide& s) {
  CellCore& core = h->cl->core;
  h->ix = s.idx[0];
  h->ixh = s.idx[1];
  h->iv = s.idx[2];
  h->ivh = s.idx[3];
  h->irho = s.idx[4];
  h->irhoh = s.idx[5];
  h->PT.p = s.pt[0];
  h->PT_b.p = s.pt[1];
  for (int d = 0; d < 3; ++d) {
    h->BUF2[d].p = s.buf2[d][0];
    h->BUF2_b[d].p = s.buf2[d][1];
  }
  core.orig.p = s.orig[0];
  core.orig_b.p = s.orig[1];
  core.sorted = s.sorted;
  core.built = s.built;
  core.up_valid = s.up_valid;
  core.rows_upper = s.rows_upper;
  h->in_cell_order = s.in_cell_order;
  core.nfull = s.nfull;
}

static GraphKey graph_key(const sph_handle* h, int32_t n, int timestepping, double tmin, double tmax) {
  GraphKey k;
  memset(&k, 0, sizeof(k));  // padding compares too
  k.n = n;
  k.timestepping = timestepping;
  k.lanes = choose_lanes(h);
  k.timing = timing_on() ? 1 : 0;
  k.dt_relative = h->dt_relative;
  k.tmin = timestepping ? tmin : 0.0;
  k.tmax = timestepping ? tmax : 0.0;
  k.prm = h->prm;
  k.prm.dt = 0.0;
  k.prm.etime = 0.0;
  k.nbr_cap = h->cl->core.nbr_cap;
  k.we_cap = h->we_cap;
  k.gen = h->cl->core.gen;
  k.at = host_side(h);
  // flags and counts the capture does not depend on (it always starts by
  // binning the caller's points) stay out of the key
  k.at.sorted = k.at.built = k.at.up_valid = k.at.in_cell_order = k.at.rows_upper = false;
  k.at.nfull = 0;
  for (int d = 0; d < 3; ++d) {
    k.user[d] = h->cl->xuser[d];
    k.user[3 + d] = h->v_u[d];
  }
  k.user[6] = h->rho_u;
  k.user[7] = h->pt_u;
  return k;
}

template <int D>
static int graph_capture(sph_handle* h, StepConst c, int32_t n, StepGraph& g) {
  CellCore& core = h->cl->core;
  // the caller's stream may be the legacy default stream, which cannot be
  // captured: record into a private stream (nothing runs there)
  if (!h->cap_stream) GC_CUDA(cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking));
  const cudaStream_t run_st = core.st;
  cudaStream_t st = h->cap_stream;
  Scal* dsc = h->scal.as<Scal>();
  const HostSide before = host_side(h);
  const unsigned long long l0 = gcsph_launch_count();
  GC_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  core.st = st;
  timer_capture_to(&g.timers);
  int rc = GCSPH_OK;
  int32_t cspmcnt = 0;
  // the step's maxima start at zero (the call's scalars are uploaded before
  // each replay) and each step's end clears them for the next; the overflow
  // flag stays set once raised
  c.reset_max = 1;
  h->keys_ready = false;
  for (int32_t it = 0; it < n && rc == GCSPH_OK; ++it) {
    c.count_reb = it + 1 < n;
    if ((rc = rebuild<D>(h, c, &dsc->ovf))) break;
    rc = enqueue_stages<D>(h, c, dsc, cspmcnt, it + 1 < n);
  }
  if (rc == GCSPH_OK) rc = finish_call<D>(h, c, dsc);
  h->keys_ready = false;
  timer_capture_to(nullptr);
  core.st = run_st;
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(st, &graph);
  const unsigned long long l1 = gcsph_launch_count();
  count_launch(-(int)(l1 - l0));  // captured, not run: each replay counts them
  if (rc == GCSPH_OK && e != cudaSuccess) rc = cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  if (rc == GCSPH_OK) {
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
  }
  if (graph) cudaGraphDestroy(graph);
  g.after = host_side(h);
  set_host_side(h, before);
  if (rc != GCSPH_OK) {
    cudaGetLastError();
    graph_free(g);
    return rc;
  }
  g.launches = (long long)(l1 - l0);
  return GCSPH_OK;
}

// GCSPH_OK with *done = false: not eligible, run the eager loop
template <int D>
static int step_graph(sph_handle* h, const StepConst& c, int32_t n, int timestepping, double tmin, double tmax,
                      int64_t* updaten_out, double* maxcdx_out, bool* done) {
  *done = false;
  CellCore& core = h->cl->core;
  if (!h->use_graphs || n < 1 || !(c.reb_thr <= 0.0) || h->in_cell_order || core.nbr_cap <= 0 ||
      h->we_cap < core.nbr_cap || core.nfull_est <= 0)
    return GCSPH_OK;
  cudaStream_t st = core.st;
  Scal* dsc = h->scal.as<Scal>();
  const GraphKey key = graph_key(h, n, timestepping, tmin, tmax);
  StepGraph* g = nullptr;
  for (StepGraph& e : h->graphs)
    if (e.exec && memcmp(&e.key, &key, sizeof(key)) == 0) g = &e;
  if (!g) {
    // least recently used slot
    g = &h->graphs[0];
    for (StepGraph& e : h->graphs)
      if (!e.exec || e.used < g->used) g = &e;
    graph_free(*g);
    g->key = key;
    if (graph_capture<D>(h, c, n, *g) != GCSPH_OK) {
      // capture is an optimisation: the eager loop runs the call
      cudaGetLastError();
      set_error("");
      return GCSPH_OK;
    }
    h->n_captures += 1;
  }
  g->used = ++h->graph_clock;
  init_scal(h, n);
  GC_CUDA(cudaMemcpyAsync(dsc, h->pin, sizeof(Scal), cudaMemcpyHostToDevice, st));
  GC_CUDA(cudaGraphLaunch(g->exec, st));
  GC_CUDA(cudaMemcpyAsync(h->pin, dsc, sizeof(Scal), cudaMemcpyDeviceToHost, st));
  GC_CUDA(cudaStreamSynchronize(st));
  count_launch((int)g->launches);
  timer_account(g->timers);
  if (h->pin->ovf) {
    // the caller's arrays are untouched; grow past the count that overflowed
    int rc;
    if ((rc = core.read_nfull())) return rc;
    if ((rc = core.grow_nbr(core.nfull))) return rc;
    if ((rc = grow_entry_arrays<D>(h))) return rc;
    core.sorted = core.built = core.up_valid = false;
    return GCSPH_OK;  // not done: the eager loop runs the call
  }
  set_host_side(h, g->after);
  h->n_replays += 1;
  h->prm.dt = h->pin->dt;
  h->prm.etime = h->pin->etime;
  double mo;
  unsigned long long bits = h->pin->maxout;
  memcpy(&mo, &bits, 8);
  if (updaten_out) *updaten_out = h->pin->nreb;
  if (maxcdx_out) *maxcdx_out = mo;
  *done = true;
  return GCSPH_OK;
}

template <int D>
static int step_impl(sph_handle* h, int32_t n, int timestepping, double tmin, double tmax, int64_t* updaten_out,
                     double* maxcdx_out) {
  StepConst c = make_const(h);
  c.timestepping = timestepping;
  c.tmin = tmin;
  c.tmax = tmax;
  c.reb_thr = 0.9 * h->prm.nui;
  c.dt_relative = h->dt_relative;
  bool done = false;
  int rc = step_graph<D>(h, c, n, timestepping, tmin, tmax, updaten_out, maxcdx_out, &done);
  if (!rc && !done) rc = step_eager<D>(h, c, n, updaten_out, maxcdx_out);
  // the call has finished on the device: the most crowded cell it binned
  // picks the in-cell ordering of the next call (large sets)
  if (!rc) rc = h->cl->core.read_popmax();
  return rc;
}

extern "C" {

int sph_create(gcl_handle* cl, const gcsph_params* prm, double* rho_dev, double* const* v_dev,
               const int32_t* ptype_dev, sph_handle** out) {
  if (!cl || !prm || !rho_dev || !ptype_dev || !out) return fail(GCSPH_EINVAL, "null argument");
  *out = nullptr;
  if (prm->gamma <= 0) return fail(GCSPH_EINVAL, "gamma must be a positive integer");
  sph_handle* h = new sph_handle();
  h->cl = cl;
  h->D = cl->core.D;
  h->N = cl->core.N;
  h->prm = *prm;
  h->rho_u = rho_dev;
  h->pt_u = ptype_dev;
  cudaStream_t st = cl->core.st;
  const int64_t N = h->N;
  const size_t nb = sizeof(double) * (size_t)N;
  int rc = GCSPH_OK;
  auto E = [&](DevBuf& b, size_t bytes, bool zero) {
    if (!rc) rc = b.ensure(bytes, st, zero);
  };
  for (int d = 0; d < h->D; ++d) {
    if (v_dev && v_dev[d]) {
      h->v_u[d] = v_dev[d];
    } else {
      E(h->vown[d], nb, true);
      h->v_u[d] = h->vown[d].as<double>();
    }
    E(h->vh_o[d], nb, false);
    E(h->xh_o[d], nb, false);
    E(h->cdx_o[d], nb, true);
    E(h->a_o[d], nb, true);
    E(h->buf2_o[d], nb, true);
    E(h->sumgW_o[d], nb, true);
    for (int b = 0; b < 2; ++b) {
      E(h->X[b][d], nb, false);
      E(h->XH[b][d], nb, false);
      E(h->V[b][d], nb, false);
      E(h->VH[b][d], nb, false);
    }
    E(h->A[d], nb, true);
    E(h->CDX[d], nb, true);
    E(h->BUF2[d], nb, true);
    E(h->BUF2_b[d], nb, true);
  }
  E(h->rhoh_o, nb, false);
  E(h->P_o, nb, true);
  E(h->drho_o, nb, true);
  E(h->sumW_o, nb, true);
  for (int b = 0; b < 2; ++b) {
    E(h->RHO[b], nb, false);
    E(h->RHOH[b], nb, false);
  }
  E(h->P1, nb, true);
  E(h->P2, nb, true);
  E(h->IR, nb, true);
  E(h->IRH, nb, true);
  E(h->PT, sizeof(int32_t) * N, false);
  E(h->PT_b, sizeof(int32_t) * N, false);
  E(h->DRHO, nb, true);
  E(h->PLAST, nb, true);
  E(h->scal, sizeof(Scal), true);
  if (!rc) {
    cudaError_t e = cudaMallocHost((void**)&h->pin, sizeof(Scal));
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMallocHost", __FILE__, __LINE__);
  }
  if (!rc) {
    // ρΔt½ = deepcopy(ρ), vΔt½ = deepcopy.(v), xΔt½ = deepcopy(points) (src/sphproblem.jl:141-143)
    cudaError_t e = cudaMemcpyAsync(h->rhoh_o.p, rho_dev, nb, cudaMemcpyDeviceToDevice, st);
    for (int d = 0; d < h->D && e == cudaSuccess; ++d) {
      e = cudaMemcpyAsync(h->vh_o[d].p, h->v_u[d], nb, cudaMemcpyDeviceToDevice, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(h->xh_o[d].p, cl->xuser[d], nb, cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "initial copies", __FILE__, __LINE__);
  }
  if (rc) {
    std::string keep = gcsph_last_error();
    sph_destroy(h);
    set_error("%s", keep.c_str());
    return rc;
  }
  *out = h;
  return GCSPH_OK;
}

void sph_destroy(sph_handle* h) {
  if (!h) return;
  if (h->cl) cudaStreamSynchronize(h->cl->core.st);
  for (StepGraph& g : h->graphs) graph_free(g);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  DevBuf* one[] = {&h->rhoh_o, &h->P_o, &h->drho_o, &h->sumW_o, &h->P1, &h->P2, &h->PT, &h->DRHO, &h->PLAST,
                   &h->We, &h->IR, &h->IRH, &h->scal, &h->RHO[0], &h->RHO[1], &h->RHOH[0], &h->RHOH[1], &h->PT_b};
  for (DevBuf* b : one) b->release();
  h->CD.release();
  h->PQ.release();
  for (int d = 0; d < 3; ++d) {
    h->CA[d].release();
    h->BUF2_b[d].release();
    h->vown[d].release();
    h->vh_o[d].release();
    h->xh_o[d].release();
    h->cdx_o[d].release();
    h->a_o[d].release();
    h->buf2_o[d].release();
    h->sumgW_o[d].release();
    h->A[d].release();
    h->CDX[d].release();
    h->BUF2[d].release();
    h->GWe[d].release();
    for (int b = 0; b < 2; ++b) {
      h->X[b][d].release();
      h->XH[b][d].release();
      h->V[b][d].release();
      h->VH[b][d].release();
    }
  }
  if (h->pin) cudaFreeHost(h->pin);
  delete h;
}

int sph_set_params(sph_handle* h, const gcsph_params* prm) {
  if (!h || !prm) return fail(GCSPH_EINVAL, "null argument");
  if (prm->gamma <= 0) return fail(GCSPH_EINVAL, "gamma must be a positive integer");
  h->prm = *prm;
  return GCSPH_OK;
}

int sph_set_graphs(sph_handle* h, int32_t on) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  h->use_graphs = on != 0;
  return GCSPH_OK;
}

int sph_set_dt_variant(sph_handle* h, int32_t relative) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  h->dt_relative = relative != 0;
  return GCSPH_OK;
}

int sph_graph_stats(const sph_handle* h, int64_t* captures, int64_t* replays) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  if (captures) *captures = h->n_captures;
  if (replays) *replays = h->n_replays;
  return GCSPH_OK;
}

int sph_set_lanes(sph_handle* h, int32_t lanes) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  if (!(lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8 || lanes == 16 || lanes == 32))
    return fail(GCSPH_EINVAL, "lanes must be 0 (auto), 1, 2, 4, 8, 16 or 32");
  h->lanes = lanes;
  return GCSPH_OK;
}

int sph_get_params(const sph_handle* h, gcsph_params* prm) {
  if (!h || !prm) return fail(GCSPH_EINVAL, "null argument");
  *prm = h->prm;
  return GCSPH_OK;
}

int sph_step(sph_handle* h, int32_t n, int timestepping, double tmin, double tmax, int64_t* updaten,
             double* maxcdx) {
  if (!h) return fail(GCSPH_EINVAL, "null handle");
  if (n < 0) return fail(GCSPH_EINVAL, "n must be >= 0");
  if (timestepping && tmin > tmax) return fail(GCSPH_EINVAL, "timelims[1] should be < timelims[2]");
  return h->D == 2 ? step_impl<2>(h, n, timestepping, tmin, tmax, updaten, maxcdx)
                   : step_impl<3>(h, n, timestepping, tmin, tmax, updaten, maxcdx);
}

int sph_get_field(sph_handle* h, int32_t field, void* dst) {
  if (!h || !dst) return fail(GCSPH_EINVAL, "null argument");
  cudaStream_t st = h->cl->core.st;
  const size_t nb = sizeof(double) * (size_t)h->N;
  const void* src[3] = {nullptr, nullptr, nullptr};
  int nvec = 1;
  size_t bytes = nb;
  switch (field) {
    case GCSPH_F_X: nvec = h->D; for (int d = 0; d < h->D; ++d) src[d] = h->cl->xuser[d]; break;
    case GCSPH_F_RHO: src[0] = h->rho_u; break;
    case GCSPH_F_V: nvec = h->D; for (int d = 0; d < h->D; ++d) src[d] = h->v_u[d]; break;
    case GCSPH_F_P: src[0] = h->P_o.p; break;
    case GCSPH_F_A: nvec = h->D; for (int d = 0; d < h->D; ++d) src[d] = h->a_o[d].p; break;
    case GCSPH_F_DRHODT: src[0] = h->drho_o.p; break;
    case GCSPH_F_RHOH: src[0] = h->rhoh_o.p; break;
    case GCSPH_F_VH: nvec = h->D; for (int d = 0; d < h->D; ++d) src[d] = h->vh_o[d].p; break;
    case GCSPH_F_XH: nvec = h->D; for (int d = 0; d < h->D; ++d) src[d] = h->xh_o[d].p; break;
    case GCSPH_F_CDX: nvec = h->D; for (int d = 0; d < h->D; ++d) src[d] = h->cdx_o[d].p; break;
    case GCSPH_F_SUMW: src[0] = h->sumW_o.p; break;
    case GCSPH_F_SUMGW: nvec = h->D; for (int d = 0; d < h->D; ++d) src[d] = h->sumgW_o[d].p; break;
    case GCSPH_F_BUF2: nvec = h->D; for (int d = 0; d < h->D; ++d) src[d] = h->buf2_o[d].p; break;
    case GCSPH_F_PTYPE: src[0] = h->pt_u; bytes = sizeof(int32_t) * (size_t)h->N; break;
    default: return fail(GCSPH_EINVAL, "unknown field %d", (int)field);
  }
  for (int d = 0; d < nvec; ++d)
    GC_CUDA(cudaMemcpyAsync((char*)dst + (size_t)d * bytes, src[d], bytes, cudaMemcpyDeviceToDevice, st));
  GC_CUDA(cudaStreamSynchronize(st));
  return GCSPH_OK;
}

}  // extern "C"
