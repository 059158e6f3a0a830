// sph_step.cuh -- types and per-pair device helpers shared by the fused
// FP64 step kernels (sph_step.cu, compiled without FMA contraction so that
// the serial row order reproduces the CPU oracle bit for bit) and the
// pair-once split-row passes (sph_once.cu, compiled with contraction).
#pragma once
#include <math.h>
#include "celllist.cuh"
#include "pf7_series.cuh"

namespace gcsph {

static constexpr int STPB = 128;

struct StepConst {
  double h, eta2, m0, rho0, ginv, DDTkh, DDTgz, P0, alpha, c0, nu, g, s, Hinv, nW, nDW;
  double fb_d, fb_r0, fb_eta2;  // fbmolforce constants of the stage being run
  // pair-once products of the constants: d𝒲/r = dWr (1 - u)^3 (u / r = H⁻¹),
  // δ-SPH's DDTkh m₀, and ∂v∂t_av!'s 2 α c₀ h m₀
  double dWr, DDTkhm0, avK;
  double twoh, pfc, hp1;        // 2h, 1.5*pi, 0.1h  (∂v∂tpF!)
  double dpc_l0inv, dpc_nW, dpc_whinv, dpc_pmin, dpc_pmax, dpc_lambda, dpc_kernlim, dpc_eta2;
  double dpc_r2cut;  // l0² (1 + 1e-6): past it u = √r² / l0 >= 1 whatever the rounding
  double xsph_c;                // 2*m0*eps
  double cfl, dt_eta2;          // Δt_stepping
  double tmin, tmax;
  int gamma, use_visc, use_pF, timestepping;
  int fold_end;    // pass B2's last block does k_step_end's work (no Δt_stepping in this call)
  int reset_max;   // the step's end clears the step's maxima for the next (captured calls: no memset node)
  double reb_thr;  // update! is due after a step whose max |cΔx| passes this (0.9 (dist - H))
  int dt_relative; // Δt_stepping's velocity term from pair-relative Δv·Δx instead of absolute v·x
  int count_reb;   // this step's decision counts toward the call's update! total
  int need_w;      // pass A stage 1 writes W: xsphcorr! or this step's cspmcorr! reads it
};

// device scalars of a running solve
struct Scal {
  double dt;
  double etime;
  unsigned long long maxcdx;  // bits of max |cΔx| of the current step
  unsigned long long amax;    // bits of max |a|
  unsigned long long vmax;    // bits of max |h v.x/(x.x+η²)|
  int ovf;                    // the neighbour CSR outgrew its buffers: this step's kernels skip
  unsigned bdone;             // blocks of pass B2 done this step (k_step_end's work in its last block)
  unsigned long long maxout;  // bits of the largest max |cΔx| of the call (stepsolve!'s second result)
  long long nreb;             // update! calls of the call (stepsolve!'s first result)
};

template <int D>
struct SArr {
  const int64_t* rs;
  const int32_t* nbr;
  const int32_t* pt;
  const int32_t* orig;
  const int* ovf;  // set: the step's kernels skip (buffers outgrown, see rebuild)
  double* x[3];
  double* v[3];
  double* rho;
  double* P1;
  double* xh[3];
  double* vh[3];
  double* rhoh;
  double* P2;
  double* ir;   // 1/ρ (FAST stage 1)
  double* irh;  // 1/ρΔt½ (FAST stage 2)
  double* We;
  double* gWe[3];
  double* a[3];
  double* drho;
  double* cdx[3];
  double* buf2[3];
  double* Plast;
  double* xo[3];
  double* xho[3];
  double* vho[3];
  double* vo[3];
  double* rhoho;
  double* rhoo;
};

template <int D>
__device__ inline double dotD(const double* a, const double* b) {
  double s = a[0] * b[0];
#pragma unroll
  for (int d = 1; d < D; ++d) s = s + a[d] * b[d];
  return s;
}

// Julia min/max propagate NaN (fmin/fmax do not)
__device__ inline double jl_min(double a, double b) { return (a != a || b != b) ? (a + b) : fmin(a, b); }
__device__ inline double jl_max(double a, double b) { return (a != a || b != b) ? (a + b) : fmax(a, b); }

// the end of a step, one thread: etime += Δt (src/sphproblem.jl:331), the
// update! decision from max |cΔx| (:325-327), the call's largest max |cΔx|,
// and with Δt_stepping the next Δt from the step's maxima
__device__ inline void step_end_body(const StepConst& c, Scal* sc) {
  const double dt = sc->dt;
  sc->etime = sc->etime + dt;
  const double mc = __longlong_as_double((long long)sc->maxcdx);
  if (sc->maxcdx > sc->maxout) sc->maxout = sc->maxcdx;
  if (c.count_reb && mc > c.reb_thr) sc->nreb += 1;
  if (c.timestepping) {
    const double amax = __longlong_as_double((long long)sc->amax);
    const double vmax = __longlong_as_double((long long)sc->vmax);
    const double dt1 = sqrt(c.h / (3.0 * amax));
    const double dt2 = c.h / (c.c0 + vmax);
    double nd = c.cfl * jl_min(dt1, dt2);
    nd = jl_min(jl_max(nd, c.tmin), c.tmax);
    sc->dt = nd;
  }
  if (c.reset_max) {
    sc->maxcdx = 0ull;
    sc->amax = 0ull;
    sc->vmax = 0ull;
  }
}

// ∂ρ∂tDDT! pair value seen from particle k (src/gpukernels_sph.jl:579-625)
template <int D>
__device__ inline double ddt_term(const StepConst& c, int ptk, int ptm, const double* dx, double r2, const double* gw,
                                  const double* dv, double rk, double rm) {
  if (!(ptk > 0 && ptm > 0)) return 0.0;
  double dot3 = -dotD<D>(dx, gw);
  double m0dot = c.m0 * dotD<D>(dv, gw);
  double s = m0dot;
  if (ptk > 1) {
    double drhopvp = c.rho0 * powfancy7th(1.0 + c.DDTgz * dx[1], c.ginv, c.gamma) - c.rho0;
    double visc_densi = c.DDTkh * ((rm - rk) - drhopvp) / (r2 + c.eta2);
    double delta = visc_densi * dot3 * c.m0 / rm;
    s += delta;
  }
  return s;
}

// all momentum terms of one pair seen from k; accumulators kept apart so the
// final sum follows the reference's kernel order (∂v∂t!, av, visc, grav, fb, pF)
template <int D>
struct Acc {
  double p[D], av[D], vi[D], fb[D], pf[D];
  __device__ void zero() {
#pragma unroll
    for (int d = 0; d < D; ++d) p[d] = av[d] = vi[d] = fb[d] = pf[d] = 0.0;
  }
};

template <int D>
__device__ inline void mom_terms(const StepConst& c, Acc<D>& A, int ptk, int ptm, const double* dx, double r2,
                                 const double* gw, const double* dv, double rk, double rm, double Pk, double Pm) {
  // ∂v∂t!, :755-772
  if (ptk * ptm > 0) {
    double Pfac = (Pk + Pm) / (rk * rm);
    double sc = -c.m0 * Pfac;
#pragma unroll
    for (int d = 0; d < D; ++d) A.p[d] += sc * gw[d];
  }
  if (ptk > 0 && ptm > 0) {
    // ∂v∂t_av!, :869-897
    double rhom = (rk + rm) * 0.5;
    double cond = dotD<D>(dv, dx);
    if (cond < 0.0) {
      double dmu = c.h * cond / (r2 + c.eta2);
      double dPi = (-c.alpha * c.c0 * dmu) / rhom;
      double sc = -dPi * c.m0;
#pragma unroll
      for (int d = 0; d < D; ++d) A.av[d] += sc * gw[d];
    }
    // ∂v∂t_visc!, :967-980
    if (c.use_visc) {
      double nuterm = 4.0 * c.nu * c.m0 * dotD<D>(dx, gw) / ((rk + rm) * (r2 + c.eta2));
#pragma unroll
      for (int d = 0; d < D; ++d) A.vi[d] += nuterm * dv[d];
    }
  }
}

// fbmolforce!, :1891-1901 (mask: exactly one side real)
template <int D>
__device__ inline void fb_term(const StepConst& c, Acc<D>& A, int ptk, int ptm, const double* dx, double r2) {
  if ((ptk > 0) == (ptm > 0)) return;
  double r = sqrt(r2);
  if (r < c.fb_r0) {
    double q = c.fb_r0 / (r + c.fb_eta2);
    double q2 = q * q, q4 = q2 * q2, q8 = q4 * q4, q12 = q8 * q4;
    double Fc = c.fb_d * (q12 - q4) / (r2 + c.fb_eta2);
#pragma unroll
    for (int d = 0; d < D; ++d) A.fb[d] += dx[d] * Fc;
  }
}

// ∂v∂tpF!, :1387-1397
template <int D>
__device__ inline void pf_term(const StepConst& c, Acc<D>& A, int ptk, int ptm, const double* dx, double r) {
  if (!(ptk > 0 && ptm > 0)) return;
  if (r < c.twoh) {
    double scos = c.s * gc_cos(c.pfc * r / c.twoh) / (r + c.hp1);
#pragma unroll
    for (int d = 0; d < D; ++d) A.pf[d] += scos * dx[d] / c.m0;
  }
}

// ---------------------------------------------------------------------------
// FAST variants (lanes > 1): the same terms with fewer FP64 divisions -- the
// FP64 pipe issues 2 thread-instructions per cycle per SM on GB300 and an IEEE
// division costs ~8 of them.  1/ρ per particle is precomputed, 1/(r²+η²) is
// shared by ∂ρ∂tDDT!, ∂v∂t_av! and ∂v∂t_visc!, 1/(ρᵢ+ρⱼ) by av and visc, and
// powfancy7th's Newton step t - t(t³ - x/t⁴)/(4t³ + 3x/t⁴) is evaluated in the
// equal form t - t(t⁷ - x)/(4t⁷ + 3x) with one division.  Each change moves a
// result by a few ulp, inside the spread the reference's own atomics give.
// ---------------------------------------------------------------------------
__device__ inline double powfancy7th_1div(double x, double ginv, int gamma) {
  if (gamma != 7) return pow(x, ginv);
  const double ax = fabs(x);
  unsigned long long bits = (unsigned long long)__double_as_longlong(ax);
  bits = 0x36cd000000000000ULL + bits / 7ULL;
  double t = copysign(__longlong_as_double((long long)bits), x);
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const double t2 = t * t;
    const double t3 = t2 * t;
    const double t7 = t3 * (t2 * t2);
    t = t - (t * (t7 - x)) / (4.0 * t7 + 3.0 * x);
  }
  return t;
}

template <int D>
__device__ inline double ddt_term_fast(const StepConst& c, int ptk, const double* dx, double inv_r2eta,
                                       const double* gw, const double* dv, double rk, double rm, double irm) {
  double dot3 = -dotD<D>(dx, gw);
  double s = c.m0 * dotD<D>(dv, gw);
  if (ptk > 1) {
    double drhopvp = c.rho0 * powfancy7th_1div(1.0 + c.DDTgz * dx[1], c.ginv, c.gamma) - c.rho0;
    double visc_densi = c.DDTkh * ((rm - rk) - drhopvp) * inv_r2eta;
    s += visc_densi * dot3 * c.m0 * irm;
  }
  return s;
}

template <int D>
__device__ inline void mom_terms_fast(const StepConst& c, Acc<D>& A, int ptk, int ptm, const double* dx,
                                      double inv_r2eta, const double* gw, const double* dv, double rk, double rm,
                                      double irk, double irm, double Pk, double Pm) {
  if (ptk * ptm > 0) {
    const double sc = -c.m0 * ((Pk + Pm) * (irk * irm));
#pragma unroll
    for (int d = 0; d < D; ++d) A.p[d] += sc * gw[d];
  }
  if (ptk > 0 && ptm > 0) {
    const double cond = dotD<D>(dv, dx);
    const bool av = cond < 0.0;
    if (av || c.use_visc) {
      const double inv_sum = 1.0 / (rk + rm);
      if (av) {
        const double dmu = c.h * cond * inv_r2eta;
        const double dPi = (-c.alpha * c.c0 * dmu) * (2.0 * inv_sum);
        const double sc = -dPi * c.m0;
#pragma unroll
        for (int d = 0; d < D; ++d) A.av[d] += sc * gw[d];
      }
      if (c.use_visc) {
        const double nuterm = 4.0 * c.nu * c.m0 * dotD<D>(dx, gw) * inv_sum * inv_r2eta;
#pragma unroll
        for (int d = 0; d < D; ++d) A.vi[d] += nuterm * dv[d];
      }
    }
  }
}

// a = ((((p + av) + visc) - g) + fb) + pF
template <int D>
__device__ inline void finish_acc(const StepConst& c, const Acc<D>& A, double* a) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double v = A.p[d] + A.av[d];
    if (c.use_visc) v = v + A.vi[d];
    v = v - (d == 1 ? c.g : 0.0);
    v = v + A.fb[d];
    if (c.use_pF) v = v + A.pf[d];
    a[d] = v;
  }
}

// ---------------------------------------------------------------------------
// Sub-warp cooperation: L lanes (1, 2, 4, 8, 16 or 32) share one particle.
// Lane l walks row entries e0+l, e0+l+L, ...; the per-lane partial sums are
// combined by a butterfly (xor offsets L/2 .. 1), after which every lane
// holds the same total.  L = 1 is the serial row order -- the order the
// oracle's scatter over its canonically ordered pair list produces -- so it
// reproduces the oracle bit for bit; L > 1 re-associates the sums (within
// the FP64 contract) and fills the GPU when particles are few.
// ---------------------------------------------------------------------------
template <int L>
__device__ inline unsigned group_mask() {
  if constexpr (L == 32) {
    return 0xffffffffu;
  } else {
    const unsigned lanew = threadIdx.x & 31u;
    return ((1u << L) - 1u) << (lanew & ~(unsigned)(L - 1));
  }
}
template <int L>
__device__ inline double group_sum(double v, unsigned gm) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) v = v + __shfl_xor_sync(gm, v, o);
  return v;
}
template <int D, int L>
__device__ inline void group_sum_acc(Acc<D>& A, const StepConst& c, unsigned gm) {
  if constexpr (L > 1) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      A.p[d] = group_sum<L>(A.p[d], gm);
      A.av[d] = group_sum<L>(A.av[d], gm);
      if (c.use_visc) A.vi[d] = group_sum<L>(A.vi[d], gm);
      A.fb[d] = group_sum<L>(A.fb[d], gm);
      if (c.use_pF) A.pf[d] = group_sum<L>(A.pf[d], gm);
    }
  }
}

// ---------------------------------------------------------------------------
// Pair-once stage passes (lanes > 1, the default).  The gather above
// evaluates every pair twice, once from each side; on GB300 the FP64 pipe is
// the bound, so here each pair is evaluated once.  Pass A: one thread per pair
// (k, m), k < m in cell order -- every thread has the same work, whatever the
// row lengths -- computes the pair and writes both sides' contributions into
// per-entry slots: slot e in k's row and slot mirror(e) in m's row.  Pass B:
// each particle sums its whole row (L lanes, fixed order -- deterministic, no
// atomics) and runs the predictor or the corrector.  Cost: one write + one
// read of (1+D) doubles per neighbour entry.
// ---------------------------------------------------------------------------
struct PairBuf {
  double* cd;             // ∂ρ/∂t contribution per neighbour entry
  double* ca[3];          // ∂v/∂t contribution per neighbour entry (gravity not included)
  int4* pq;               // (k, m, e, mirror(e)) of every pair, k < m (mirror -1: stage 1 finds it)
  const int64_t* npair;   // number of pairs (device scalar)
};

// ---------------------------------------------------------------------------
// Pair-once arithmetic.  The FP64 pipe is the bound of pass A (2 FP64
// thread-instructions per cycle per SM on GB300), so its compares run on the
// integer pipe over the bit patterns, and its reciprocals and its root are
// Newton-Raphson iterations from the hardware's approximate reciprocal and
// reciprocal square root (rcp.approx / rsqrt.approx .f64, about 2^-22
// relative): two steps each, quadratic convergence, a result within a few
// ulp -- fewer FP64 instructions than the IEEE-rounded sequences, inside the
// FP64 contract this path is held to.
// ---------------------------------------------------------------------------
__device__ inline long long dbits(double x) { return __double_as_longlong(x); }
constexpr long long ONE_BITS = 0x3FF0000000000000LL;  // bits of 1.0
// x < 0.0 exactly as the FP compare (-0.0 and NaN are not), on the integer pipe
__device__ inline bool neg_int(double x) {
  return (unsigned long long)dbits(x) - 0x8000000000000001ull < 0x7FF0000000000000ull;
}

// 1/x, x normal (Newton-Raphson: y <- y + y (1 - x y))
__device__ inline double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

// sqrt(x), x normal and positive (Newton-Raphson on 1/sqrt(x):
// y <- y + y (1/2 - (x/2) y^2), then x y)
__device__ inline double sqrt_nr(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double hx = 0.5 * x;
  double e = fma(-hx, y * y, 0.5);
  y = fma(y, e, y);
  e = fma(-hx, y * y, 0.5);
  y = fma(y, e, y);
  return x * y;
}

// powfancy7th(x) - 1 for x = 1 + eps, src/gpukernels_sph.jl:499-515.  Where
// |eps| <= PF7_EPS_MAX the exact Taylor series of that iteration's output
// (gen_pf7_series.py, bias included) replaces its two divisions, and where
// |eps| <= PF7_EPS_SHORT its first PF7_SHORT_N terms do; elsewhere the
// iteration itself runs.  eps is taken as (1 + eps) - 1, the argument the
// reference's rounded x carries.  Callers form ρ0 (1 + r) - ρ0 as the
// reference forms ρ0 t - ρ0: 1 + r rounds to the t the iteration returns.
__device__ inline double pf7m1_fast(double eps_in, double ginv, int gamma) {
  const double x = 1.0 + eps_in;
  const double e = x - 1.0;  // exact for x in [0.5, 2]
  const long long ae = dbits(e) & 0x7FFFFFFFFFFFFFFFLL;
  static_assert(PF7_UP_N == PF7_LO_N, "series lengths");
  if (gamma == 7 && ae <= dbits(PF7_EPS_MAX)) {
    const double cu[PF7_UP_N] = PF7_UP_C;
    const double cl[PF7_LO_N] = PF7_LO_C;
    const bool up = dbits(e) >= 0;
    double r;
    if (ae <= dbits(PF7_EPS_SHORT)) {
      r = up ? cu[PF7_SHORT_N - 1] : cl[PF7_SHORT_N - 1];
#pragma unroll
      for (int i = PF7_SHORT_N - 2; i >= 0; --i) r = fma(r, e, up ? cu[i] : cl[i]);
    } else {
      r = up ? cu[PF7_UP_N - 1] : cl[PF7_UP_N - 1];
#pragma unroll
      for (int i = PF7_UP_N - 2; i >= 0; --i) r = fma(r, e, up ? cu[i] : cl[i]);
    }
    return r;
  }
  return powfancy7th_1div(x, ginv, gamma) - 1.0;
}

// all momentum terms of one pair (FAST expressions), summed into f
template <int D>
__device__ inline void pair_force_fast(const StepConst& c, int ptk, int ptm, const double* dx, double r2,
                                       double inv_r2eta, const double* gw, const double* dv, double rk, double rm,
                                       double irk, double irm, double Pk, double Pm, double* f) {
  Acc<D> A;
  A.zero();
  mom_terms_fast<D>(c, A, ptk, ptm, dx, inv_r2eta, gw, dv, rk, rm, irk, irm, Pk, Pm);
#pragma unroll
  for (int d = 0; d < D; ++d) f[d] = (A.p[d] + A.av[d]) + (c.use_visc ? A.vi[d] : 0.0);
}

template <int D, int STAGE>
__device__ inline void pair_tail_terms(const StepConst& c, int ptk, int ptm, const double* dxf, const double* dx,
                                       double r, double* f) {
  Acc<D> A;
  A.zero();
  fb_term<D>(c, A, ptk, ptm, dxf, dotD<D>(dxf, dxf));
  if (c.use_pF) pf_term<D>(c, A, ptk, ptm, dx, r);
#pragma unroll
  for (int d = 0; d < D; ++d) f[d] = (f[d] + A.fb[d]) + (c.use_pF ? A.pf[d] : 0.0);
}

// row sums of the per-entry contributions of particle k, L lanes
template <int D, int L>
__device__ inline void row_sums(const SArr<D>& S, const PairBuf& B, int64_t k, int lane, unsigned gm, double& drho,
                                double* a) {
  drho = 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) a[d] = 0.0;
  const int64_t e0 = S.rs[k], e1 = S.rs[k + 1];
  int64_t e = e0 + lane;
  // four entries' loads in flight at a time; each sum still adds its
  // entries in row order
  for (; e + 3 * L < e1; e += 4 * L) {
    double cv[4], av[4][D];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      cv[j] = B.cd[e + j * L];
#pragma unroll
      for (int d = 0; d < D; ++d) av[j][d] = B.ca[d][e + j * L];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      drho += cv[j];
#pragma unroll
      for (int d = 0; d < D; ++d) a[d] += av[j][d];
    }
  }
  for (; e < e1; e += L) {
    drho += B.cd[e];
#pragma unroll
    for (int d = 0; d < D; ++d) a[d] += B.ca[d][e];
  }
  drho = group_sum<L>(drho, gm);
#pragma unroll
  for (int d = 0; d < D; ++d) a[d] = group_sum<L>(a[d], gm);
}


// pair-once passes (sph_once.cu): pass A over the device-side pair count,
// one block per SM; pass B (row sums + predictor / corrector) with L lanes
// per particle, 32 particles per block
template <int D>
int launch_pairA(int stage, cudaStream_t st, const StepConst& c, const SArr<D>& S, const PairBuf& B);
// The next step's binning started by pass B2 (update! every step): each
// particle's cell key and arrival slot from its new position, and, in the
// last block, the cell starts (CellCore::sort with keys_ready goes on from
// there).  key == nullptr: none.
struct NextBin {
  int32_t* key;
  int32_t* slot;
  int32_t* count;      // zero on entry, zero again on exit
  int32_t* cellstart;
  Grid g;
};
template <int D>
int launch_pairB(int stage, int L, int64_t N, cudaStream_t st, const StepConst& c, Scal* sc, const SArr<D>& S,
                 const PairBuf& B, const NextBin* nb = nullptr);

}  // namespace gcsph
