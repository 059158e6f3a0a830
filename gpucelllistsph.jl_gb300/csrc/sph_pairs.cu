// sph_pairs.cu -- the reference's exported kernel functions as C-ABI calls.
//
// Each entry point takes the caller's pair list (1-based (i,j), rows with
// i == 0 skipped) and caller arrays in original particle order, and follows the
// reference kernel of the same name (src/gpukernels_sph.jl): one thread per
// pair, FP64 atomics into both particles.  These are the drop-in for users who
// call the kernels one by one; stepsolve! itself runs the fused gather path in
// sph_step.cu.
#include <math.h>
#include "gcsph_common.cuh"

namespace gcsph {

static constexpr int PTPB = 256;

struct V3 {
  const double* p[3];
};
struct W3 {
  double* p[3];
};

static int vec_in(int D, const double* const* src, V3* out, const char* name) {
  if (!src) return fail(GCSPH_EINVAL, "null %s", name);
  for (int d = 0; d < 3; ++d) out->p[d] = nullptr;
  for (int d = 0; d < D; ++d) {
    if (!src[d]) return fail(GCSPH_EINVAL, "null %s[%d]", name, d + 1);
    out->p[d] = src[d];
  }
  return GCSPH_OK;
}
static int vec_out(int D, double* const* src, W3* out, const char* name) {
  if (!src) return fail(GCSPH_EINVAL, "null %s", name);
  for (int d = 0; d < 3; ++d) out->p[d] = nullptr;
  for (int d = 0; d < D; ++d) {
    if (!src[d]) return fail(GCSPH_EINVAL, "null %s[%d]", name, d + 1);
    out->p[d] = src[d];
  }
  return GCSPH_OK;
}

template <int D>
__device__ inline double dotp(const double* a, const double* b) {
  double s = a[0] * b[0];
#pragma unroll
  for (int d = 1; d < D; ++d) s = s + a[d] * b[d];
  return s;
}

__device__ inline bool pair_at(const int32_t* pairs, int64_t p, int64_t* i, int64_t* j) {
  int32_t a = pairs[2 * p], b = pairs[2 * p + 1];
  *i = (int64_t)a - 1;
  *j = (int64_t)b - 1;
  return a != 0;
}

// kernel_sphW! (:84-100) and kernel_sph∇W! (:196-213)
template <int D, int GRAD>
__global__ void k_fn_w(int64_t P, const int32_t* __restrict__ pairs, V3 x, double Hinv, double nn,
                       double* __restrict__ W, W3 gW) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  double dx[D];
#pragma unroll
  for (int d = 0; d < D; ++d) dx[d] = x.p[d][i] - x.p[d][j];
  double r = sqrt(dotp<D>(dx, dx));
  double u = r * Hinv;
  if (GRAD) {
    double dwk_r = wc2_dw(u, nn) / r;
#pragma unroll
    for (int d = 0; d < D; ++d) gW.p[d][p] = dx[d] * dwk_r;
  } else {
    W[p] = wc2_w(u, nn);
  }
}

// kernel_sph∑W! (:139-156), kernel_sph∑∇W! (:332-359)
template <int D, int GRAD>
__global__ void k_fn_sumw(int64_t P, const int32_t* __restrict__ pairs, V3 x, double Hinv, double nn,
                          const int32_t* __restrict__ pt, double* __restrict__ sumW, W3 sg) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if ((pt[i] > 0) != (pt[j] > 0)) return;
  double dx[D];
#pragma unroll
  for (int d = 0; d < D; ++d) dx[d] = x.p[d][i] - x.p[d][j];
  double r = sqrt(dotp<D>(dx, dx));
  double u = r * Hinv;
  if (GRAD) {
    double dwk_r = wc2_dw(u, nn) / r;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double g = dx[d] * dwk_r;
      atomicAdd(&sg.p[d][i], g);
      atomicAdd(&sg.p[d][j], -g);
    }
  } else {
    double w = wc2_w(u, nn);
    atomicAdd(&sumW[i], w);
    atomicAdd(&sumW[j], w);
  }
}

// kernel_∂ρ∂tDDT! (:571-631)
template <int D>
__global__ void k_fn_ddt(int64_t P, const int32_t* __restrict__ pairs, V3 gW, const double* __restrict__ rho, V3 v,
                         V3 x, double eta2, double m0, double rho0, double ginv, int gamma, double DDTkh, double DDTgz,
                         const int32_t* __restrict__ pt, double* __restrict__ out) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int32_t a = pairs[2 * p], b = pairs[2 * p + 1];
  if (!(a > 0)) return;
  int64_t i = a - 1, j = b - 1;
  if (!(pt[i] > 0 && pt[j] > 0)) return;
  double dx[D], dv[D], gw[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dx[d] = x.p[d][i] - x.p[d][j];
    dv[d] = v.p[d][i] - v.p[d][j];
    gw[d] = gW.p[d][p];
  }
  double r2 = dotp<D>(dx, dx);
  double ri = rho[i], rj = rho[j];
  double dot3 = -dotp<D>(dx, gw);
  double m0dot = m0 * dotp<D>(dv, gw);
  double si = m0dot, sj = m0dot;
  if (pt[i] > 1) {
    double drhopvp = rho0 * powfancy7th(1.0 + DDTgz * dx[1], ginv, gamma) - rho0;
    double vd = DDTkh * ((rj - ri) - drhopvp) / (r2 + eta2);
    si += vd * dot3 * m0 / rj;
  }
  atomicAdd(&out[i], si);
  if (pt[j] > 1) {
    double drhopvn = rho0 * powfancy7th(1.0 - DDTgz * dx[1], ginv, gamma) - rho0;
    double vd = DDTkh * ((ri - rj) - drhopvn) / (r2 + eta2);
    sj += vd * dot3 * m0 / ri;
  }
  atomicAdd(&out[j], sj);
}

__global__ void k_fn_pressure(int64_t N, const double* __restrict__ rho, int gamma, double rho0, double P0,
                              const int32_t* __restrict__ pt, double* __restrict__ P) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) P[i] = eos(rho[i], gamma, rho0, P0, pt[i]);
}

template <int D>
__device__ inline void scatter_pm(W3 a, int64_t i, int64_t j, const double* f) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    atomicAdd(&a.p[d][i], f[d]);
    atomicAdd(&a.p[d][j], -f[d]);
  }
}

// kernel_∂v∂t! (:750-776)
template <int D>
__global__ void k_fn_dvdt(int64_t P, const int32_t* __restrict__ pairs, V3 gW, const double* __restrict__ Pr,
                          double m0, const double* __restrict__ rho, const int32_t* __restrict__ pt, W3 a) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if (!(pt[i] * pt[j] > 0)) return;
  double Pfac = (Pr[i] + Pr[j]) / (rho[i] * rho[j]);
  double s = -m0 * Pfac;
  double f[D];
#pragma unroll
  for (int d = 0; d < D; ++d) f[d] = s * gW.p[d][p];
  scatter_pm<D>(a, i, j, f);
}

// kernel_∂v∂t_av! (:863-901)
template <int D>
__global__ void k_fn_av(int64_t P, const int32_t* __restrict__ pairs, V3 gW, V3 x, double h, double eta2,
                        const double* __restrict__ rho, double alpha, V3 v, double c0, double m0,
                        const int32_t* __restrict__ pt, W3 a) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if (!(pt[i] > 0 && pt[j] > 0)) return;
  double dx[D], dv[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dx[d] = x.p[d][i] - x.p[d][j];
    dv[d] = v.p[d][i] - v.p[d][j];
  }
  double r2 = dotp<D>(dx, dx);
  double rhom = (rho[i] + rho[j]) * 0.5;
  double cond = dotp<D>(dv, dx);
  if (cond < 0.0) {
    double dmu = h * cond / (r2 + eta2);
    double dPi = (-alpha * c0 * dmu) / rhom;
    double s = -dPi * m0;
    double f[D];
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = s * gW.p[d][p];
    scatter_pm<D>(a, i, j, f);
  }
}

// kernel_∂v∂t_visc! (:962-991)
template <int D>
__global__ void k_fn_visc(int64_t P, const int32_t* __restrict__ pairs, V3 gW, V3 v, const double* __restrict__ rho,
                          V3 x, double eta2, double m0, double nu, const int32_t* __restrict__ pt, W3 a) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if (!(pt[i] > 0 && pt[j] > 0)) return;
  double dx[D], dv[D], gw[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dx[d] = x.p[d][i] - x.p[d][j];
    dv[d] = v.p[d][i] - v.p[d][j];
    gw[d] = gW.p[d][p];
  }
  double r2 = dotp<D>(dx, dx);
  double nuterm = 4.0 * nu * m0 * dotp<D>(dx, gw) / ((rho[i] + rho[j]) * (r2 + eta2));
  double f[D];
#pragma unroll
  for (int d = 0; d < D; ++d) f[d] = nuterm * dv[d];
  scatter_pm<D>(a, i, j, f);
}

template <int D>
__global__ void k_fn_grav(int64_t N, double g, W3 a) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
#pragma unroll
  for (int d = 0; d < D; ++d) a.p[d][i] = a.p[d][i] - (d == 1 ? g : 0.0);
}

// kernel_fbmolforce! (:1885-1913)
template <int D>
__global__ void k_fn_fbmol(int64_t P, const int32_t* __restrict__ pairs, V3 x, double dd, double r0, double eta2,
                           const int32_t* __restrict__ pt, W3 a) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if ((pt[i] > 0) == (pt[j] > 0)) return;
  double dx[D];
#pragma unroll
  for (int d = 0; d < D; ++d) dx[d] = x.p[d][i] - x.p[d][j];
  double r2 = dotp<D>(dx, dx);
  double r = sqrt(r2);
  if (r < r0) {
    double q = r0 / (r + eta2);
    double q2 = q * q, q4 = q2 * q2, q8 = q4 * q4, q12 = q8 * q4;
    double Fc = dd * (q12 - q4) / (r2 + eta2);
    double f[D];
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = dx[d] * Fc;
    scatter_pm<D>(a, i, j, f);
  }
}

// kernel_∂v∂tpF! (:1382-1409)
template <int D>
__global__ void k_fn_pF(int64_t P, const int32_t* __restrict__ pairs, V3 x, double s, double h, double m0,
                        const int32_t* __restrict__ pt, W3 a) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if (!(pt[i] > 0 && pt[j] > 0)) return;
  double dx[D];
#pragma unroll
  for (int d = 0; d < D; ++d) dx[d] = x.p[d][i] - x.p[d][j];
  double r = sqrt(dotp<D>(dx, dx));
  if (r < 2.0 * h) {
    double scos = s * gc_cos((1.5 * GCSPH_PI64) * r / (2.0 * h)) / (r + 0.1 * h);
    double f[D];
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = scos * dx[d] / m0;
    scatter_pm<D>(a, i, j, f);
  }
}

__global__ void k_fn_update_rho(int64_t N, double* __restrict__ rho, const double* __restrict__ drho, double dt,
                                double rho0, const int32_t* __restrict__ pt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double r = rho[i] + drho[i] * dt;
  if (r < rho0 && pt[i] < 0) r = rho0;
  rho[i] = r;
}

template <int D>
__global__ void k_fn_update_v(int64_t N, W3 v, V3 a, double dt, const int32_t* __restrict__ pt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || !(pt[i] > 1)) return;
#pragma unroll
  for (int d = 0; d < D; ++d) v.p[d][i] = v.p[d][i] + a.p[d][i] * dt;
}

template <int D>
__global__ void k_fn_update_x(int64_t N, W3 x, V3 v, double dt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
#pragma unroll
  for (int d = 0; d < D; ++d) x.p[d][i] = x.p[d][i] + v.p[d][i] * dt;
}

// kernel_symplectic_update! (:1204-1245)
template <int D>
__global__ void k_fn_symplectic(int64_t N, double* __restrict__ rho, double* __restrict__ rhoh, W3 v, W3 vh, W3 x,
                                W3 xh, const double* __restrict__ drho, V3 a, double dt, W3 cdx, double rho0,
                                const int32_t* __restrict__ pt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double epsi = -(drho[i] / rhoh[i]) * dt;
  double rv = rho[i] * (2.0 - epsi) / (2.0 + epsi);
  if (rv < rho0 && pt[i] <= 1) rv = rho0;
  rhoh[i] = rv;
  rho[i] = rv;
  double ml = pt[i] > 1 ? 1.0 : 0.0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double vv = v.p[d][i];
    double nv = vv + a.p[d][i] * dt * ml;
    vh.p[d][i] = nv;
    v.p[d][i] = nv;
    double ddx = (vv + nv) * 0.5 * dt;
    cdx.p[d][i] = cdx.p[d][i] + ddx;
    double xv = x.p[d][i] + ddx;
    xh.p[d][i] = xv;
    x.p[d][i] = xv;
  }
}

__device__ inline double jmin(double a, double b) { return (a != a || b != b) ? (a + b) : fmin(a, b); }
__device__ inline double jmax(double a, double b) { return (a != a || b != b) ? (a + b) : fmax(a, b); }

// kernel_dpcreg! (:1500-1553)
template <int D>
__global__ void k_fn_dpc(int64_t P, W3 buf, V3 v, const double* __restrict__ rho, const double* __restrict__ Pr,
                         const int32_t* __restrict__ pairs, V3 x, double l0inv, double nW, double whinv, double Pmin,
                         double Pmax, double dt, double lambda, double kernlim, double eta2,
                         const int32_t* __restrict__ pt) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if (!(pt[i] > 0 && pt[j] > 0)) return;
  double dx[D], dv[D], f[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dx[d] = x.p[d][i] - x.p[d][j];
    dv[d] = v.p[d][i] - v.p[d][j];
  }
  double ri = rho[i], rj = rho[j];
  double r2 = dotp<D>(dx, dx);
  double r = sqrt(r2);
  double u = r * l0inv;
  double w = wc2_w(u, nW);
  double chi = sqrt(w * whinv);
  double k = u < kernlim ? 1.0 : chi;
  double Pb = chi * jmax(jmin(lambda * fabs(Pr[i] + Pr[j]), lambda * Pmax), Pmin);
  double vr = dotp<D>(dv, dx);
  if (vr < 0.0) {
    double vrdr = vr / (r2 + eta2);
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = k * (-vrdr * dx[d]);
  } else {
    double tvar = 2.0 * dt * Pb / ((ri + rj) * (r2 + eta2));
#pragma unroll
    for (int d = 0; d < D; ++d) f[d] = tvar * dx[d];
  }
  scatter_pm<D>(buf, i, j, f);
}

template <int D>
__global__ void k_fn_update_dpc(int64_t N, W3 v, W3 x, V3 buf, double dt, const int32_t* __restrict__ pt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || !(pt[i] > 1)) return;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    v.p[d][i] = v.p[d][i] + buf.p[d][i];
    x.p[d][i] = x.p[d][i] + buf.p[d][i] * dt;
  }
}

// kernel_xsphcorr! (:1757-1779)
template <int D>
__global__ void k_fn_xsph(int64_t P, W3 buf, const int32_t* __restrict__ pairs, const double* __restrict__ W,
                          const double* __restrict__ rho, V3 v, double m0, double eps, const int32_t* __restrict__ pt) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if (!(pt[i] > 1 && pt[j] > 1)) return;
  double xs = 2.0 * m0 * eps * W[p] / (rho[i] + rho[j]);
  double f[D];
#pragma unroll
  for (int d = 0; d < D; ++d) f[d] = (v.p[d][j] - v.p[d][i]) * xs;
  scatter_pm<D>(buf, i, j, f);
}

template <int D>
__global__ void k_fn_update_xsph(int64_t N, W3 x, V3 buf, double dt, const int32_t* __restrict__ pt) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || !(pt[i] > 1)) return;
#pragma unroll
  for (int d = 0; d < D; ++d) x.p[d][i] = x.p[d][i] + buf.p[d][i] * dt;
}

// kernel_cspmcorr_1! / _2! (:1693-1719)
__global__ void k_fn_cspm1(int64_t P, double* __restrict__ s1, double* __restrict__ s2, const double* __restrict__ W,
                           const double* __restrict__ rho, double m0, const int32_t* __restrict__ pairs,
                           const int32_t* __restrict__ pt) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P) return;
  int64_t i, j;
  if (!pair_at(pairs, p, &i, &j)) return;
  if (!(pt[i] > 0 && pt[j] > 0)) return;
  double w = W[p];
  atomicAdd(&s1[i], m0 * w);
  atomicAdd(&s2[i], w * m0 / rho[j]);
  atomicAdd(&s1[j], m0 * w);
  atomicAdd(&s2[j], w * m0 / rho[i]);
}
__global__ void k_fn_cspm2(int64_t N, double* __restrict__ rho, const double* __restrict__ s1,
                           const double* __restrict__ s2) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double nr = s1[i] / s2[i];
  if (!isnan(nr)) rho[i] = nr;
}

// kernel_Δt_stepping_norm! / kernel_Δt_stepping! + the two maxima
template <int D>
__global__ void k_fn_dt(int64_t N, V3 a, V3 v, V3 x, double h, double eta2, unsigned long long* out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double am = 0.0, vm = 0.0;
  if (i < N) {
    double av[D], vv[D], pp[D];
#pragma unroll
    for (int d = 0; d < D; ++d) { av[d] = a.p[d][i]; vv[d] = v.p[d][i]; pp[d] = x.p[d][i]; }
    am = sqrt(dotp<D>(av, av));
    vm = fabs(h * dotp<D>(vv, pp) / (dotp<D>(pp, pp) + eta2));
  }
  am = warp_max(am);
  vm = warp_max(vm);
  if ((threadIdx.x & 31) == 0) {
    atomic_max_pos(&out[0], am);
    atomic_max_pos(&out[1], vm);
  }
}

}  // namespace gcsph

using namespace gcsph;

#define CHECK_D(D) \
  if ((D) != 2 && (D) != 3) return fail(GCSPH_EINVAL, "wrong dimention: D=%d (2 or 3)", (int)(D))
#define CHECK_PAIRS(P, pairs) \
  if ((P) < 0 || ((P) > 0 && !(pairs))) return fail(GCSPH_EINVAL, "bad pair list")
#define FINISH(st)                                \
  do {                                            \
    GC_LAUNCHED();                                \
    GC_CUDA(cudaStreamSynchronize((st)));         \
    return GCSPH_OK;                              \
  } while (0)
#define DISPATCH(D, KER, GRID, ST, ...)                                  \
  do {                                                                   \
    if ((D) == 2) KER<2><<<(GRID), PTPB, 0, (ST)>>>(__VA_ARGS__);        \
    else KER<3><<<(GRID), PTPB, 0, (ST)>>>(__VA_ARGS__);                 \
  } while (0)

extern "C" {

double gcsph_dpckernlim(int32_t D) {
  // find_zero(x -> 1 - W(k, x, 1), 0.5): bisection on [0, 1] to adjacent doubles
  double nW = D == 2 ? wc2_norm_w<2>(1.0) : wc2_norm_w<3>(1.0);
  double lo = 0.0, hi = 1.0;
  double flo = 1.0 - wc2_w(lo, nW);
  for (int it = 0; it < 2000; ++it) {
    double mid = lo + (hi - lo) * 0.5;
    if (mid <= lo || mid >= hi) break;
    double fm = 1.0 - wc2_w(mid, nW);
    if (fm == 0.0) return mid;
    if ((fm < 0.0) == (flo < 0.0)) {
      lo = mid;
      flo = fm;
    } else {
      hi = mid;
    }
  }
  double fl = fabs(1.0 - wc2_w(lo, nW)), fh = fabs(1.0 - wc2_w(hi, nW));
  return fl <= fh ? lo : hi;
}

int gcsph_sphW(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* x_dev, double Hinv,
               double* W, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 x;
  int rc = vec_in(D, x_dev, &x, "x");
  if (rc) return rc;
  if (!W) return fail(GCSPH_EINVAL, "null W");
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double nn = D == 2 ? wc2_norm_w<2>(Hinv) : wc2_norm_w<3>(Hinv);
  W3 none{};
  if (D == 2) k_fn_w<2, 0><<<nblocks(P, PTPB), PTPB, 0, st>>>(P, pairs, x, Hinv, nn, W, none);
  else k_fn_w<3, 0><<<nblocks(P, PTPB), PTPB, 0, st>>>(P, pairs, x, Hinv, nn, W, none);
  (void)N;
  FINISH(st);
}

int gcsph_sphgradW(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* x_dev, double Hinv,
                   double* const* gW_dev, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 x;
  W3 g;
  int rc = vec_in(D, x_dev, &x, "x");
  if (!rc) rc = vec_out(D, gW_dev, &g, "gradW");
  if (rc) return rc;
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double nn = D == 2 ? wc2_norm_dw<2>(Hinv) : wc2_norm_dw<3>(Hinv);
  if (D == 2) k_fn_w<2, 1><<<nblocks(P, PTPB), PTPB, 0, st>>>(P, pairs, x, Hinv, nn, nullptr, g);
  else k_fn_w<3, 1><<<nblocks(P, PTPB), PTPB, 0, st>>>(P, pairs, x, Hinv, nn, nullptr, g);
  (void)N;
  FINISH(st);
}

int gcsph_sphsumW(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* x_dev, double Hinv,
                  const int32_t* pt, double* sumW, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 x;
  int rc = vec_in(D, x_dev, &x, "x");
  if (rc) return rc;
  if (!pt || !sumW) return fail(GCSPH_EINVAL, "null argument");
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double nn = D == 2 ? wc2_norm_w<2>(Hinv) : wc2_norm_w<3>(Hinv);
  W3 none{};
  if (D == 2) k_fn_sumw<2, 0><<<nblocks(P, PTPB), PTPB, 0, st>>>(P, pairs, x, Hinv, nn, pt, sumW, none);
  else k_fn_sumw<3, 0><<<nblocks(P, PTPB), PTPB, 0, st>>>(P, pairs, x, Hinv, nn, pt, sumW, none);
  (void)N;
  FINISH(st);
}

int gcsph_sphsumgradW(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* x_dev, double Hinv,
                      const int32_t* pt, double* const* sumgW_dev, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 x;
  W3 g;
  int rc = vec_in(D, x_dev, &x, "x");
  if (!rc) rc = vec_out(D, sumgW_dev, &g, "sumgradW");
  if (rc) return rc;
  if (!pt) return fail(GCSPH_EINVAL, "null ptype");
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double nn = D == 2 ? wc2_norm_dw<2>(Hinv) : wc2_norm_dw<3>(Hinv);
  if (D == 2) k_fn_sumw<2, 1><<<nblocks(P, PTPB), PTPB, 0, st>>>(P, pairs, x, Hinv, nn, pt, nullptr, g);
  else k_fn_sumw<3, 1><<<nblocks(P, PTPB), PTPB, 0, st>>>(P, pairs, x, Hinv, nn, pt, nullptr, g);
  (void)N;
  FINISH(st);
}

int gcsph_drhodt_ddt(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* gW_dev,
                     const double* rho, const double* const* v_dev, const double* const* x_dev, double h, double m0,
                     double rho0, double c0, int32_t gamma, double g, double delta, const int32_t* pt, double* out,
                     void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 gw, v, x;
  int rc = vec_in(D, gW_dev, &gw, "gradW");
  if (!rc) rc = vec_in(D, v_dev, &v, "v");
  if (!rc) rc = vec_in(D, x_dev, &x, "x");
  if (rc) return rc;
  if (!rho || !pt || !out) return fail(GCSPH_EINVAL, "null argument");
  if (gamma <= 0) return fail(GCSPH_EINVAL, "gamma must be a positive integer");
  cudaStream_t st = (cudaStream_t)stream;
  GC_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)N, st));
  double eta2 = (0.1 * h) * (0.1 * h);
  double ginv = 1.0 / (double)gamma;
  double DDTkh = 2.0 * h * delta * c0;
  double Cb = (c0 * c0 * rho0) * ginv;
  double DDTgz = rho0 * g / Cb;
  if (P > 0) {
    DISPATCH(D, k_fn_ddt, nblocks(P, PTPB), st, P, pairs, gw, rho, v, x, eta2, m0, rho0, ginv, gamma, DDTkh, DDTgz,
             pt, out);
    GC_LAUNCHED();
  }
  GC_CUDA(cudaStreamSynchronize(st));
  return GCSPH_OK;
}

int gcsph_pressure(int64_t N, const double* rho, double c0, int32_t gamma, double rho0, const int32_t* pt, double* P,
                   void* stream) {
  if (!rho || !pt || !P) return fail(GCSPH_EINVAL, "null argument");
  if (gamma <= 0) return fail(GCSPH_EINVAL, "gamma must be a positive integer");
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double P0 = c0 * c0 * rho0 / (double)gamma;
  k_fn_pressure<<<nblocks(N, PTPB), PTPB, 0, st>>>(N, rho, gamma, rho0, P0, pt, P);
  FINISH(st);
}

int gcsph_dvdt(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* gW_dev, const double* Pr,
               double m0, const double* rho, const int32_t* pt, double* const* a_dev, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 gw;
  W3 a;
  int rc = vec_in(D, gW_dev, &gw, "gradW");
  if (!rc) rc = vec_out(D, a_dev, &a, "a");
  if (rc) return rc;
  if (!Pr || !rho || !pt) return fail(GCSPH_EINVAL, "null argument");
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DISPATCH(D, k_fn_dvdt, nblocks(P, PTPB), st, P, pairs, gw, Pr, m0, rho, pt, a);
  (void)N;
  FINISH(st);
}

int gcsph_dvdt_av(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* gW_dev,
                  const double* const* x_dev, double h, const double* rho, double alpha, const double* const* v_dev,
                  double c0, double m0, const int32_t* pt, double* const* a_dev, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 gw, x, v;
  W3 a;
  int rc = vec_in(D, gW_dev, &gw, "gradW");
  if (!rc) rc = vec_in(D, x_dev, &x, "x");
  if (!rc) rc = vec_in(D, v_dev, &v, "v");
  if (!rc) rc = vec_out(D, a_dev, &a, "a");
  if (rc) return rc;
  if (!rho || !pt) return fail(GCSPH_EINVAL, "null argument");
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double eta2 = (0.1 * h) * (0.1 * h);
  DISPATCH(D, k_fn_av, nblocks(P, PTPB), st, P, pairs, gw, x, h, eta2, rho, alpha, v, c0, m0, pt, a);
  (void)N;
  FINISH(st);
}

int gcsph_dvdt_visc(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* gW_dev,
                    const double* const* v_dev, const double* rho, const double* const* x_dev, double h, double m0,
                    double nu, const int32_t* pt, double* const* a_dev, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 gw, x, v;
  W3 a;
  int rc = vec_in(D, gW_dev, &gw, "gradW");
  if (!rc) rc = vec_in(D, x_dev, &x, "x");
  if (!rc) rc = vec_in(D, v_dev, &v, "v");
  if (!rc) rc = vec_out(D, a_dev, &a, "a");
  if (rc) return rc;
  if (!rho || !pt) return fail(GCSPH_EINVAL, "null argument");
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double eta2 = (0.1 * h) * (0.1 * h);
  DISPATCH(D, k_fn_visc, nblocks(P, PTPB), st, P, pairs, gw, v, rho, x, eta2, m0, nu, pt, a);
  (void)N;
  FINISH(st);
}

int gcsph_addgrav(int32_t D, int64_t N, double g, double* const* a_dev, void* stream) {
  CHECK_D(D);
  W3 a;
  int rc = vec_out(D, a_dev, &a, "a");
  if (rc) return rc;
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DISPATCH(D, k_fn_grav, nblocks(N, PTPB), st, N, g, a);
  FINISH(st);
}

int gcsph_fbmolforce(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* x_dev, double d,
                     double r0, const int32_t* pt, double* const* a_dev, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 x;
  W3 a;
  int rc = vec_in(D, x_dev, &x, "x");
  if (!rc) rc = vec_out(D, a_dev, &a, "a");
  if (rc) return rc;
  if (!pt) return fail(GCSPH_EINVAL, "null ptype");
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  double eta2 = 0.01 * (r0 * r0);
  DISPATCH(D, k_fn_fbmol, nblocks(P, PTPB), st, P, pairs, x, d, r0, eta2, pt, a);
  (void)N;
  FINISH(st);
}

int gcsph_dvdt_pF(int32_t D, int64_t N, int64_t P, const int32_t* pairs, const double* const* x_dev, double s,
                  double h, double m0, const int32_t* pt, double* const* a_dev, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  V3 x;
  W3 a;
  int rc = vec_in(D, x_dev, &x, "x");
  if (!rc) rc = vec_out(D, a_dev, &a, "a");
  if (rc) return rc;
  if (!pt) return fail(GCSPH_EINVAL, "null ptype");
  if (P == 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DISPATCH(D, k_fn_pF, nblocks(P, PTPB), st, P, pairs, x, s, h, m0, pt, a);
  (void)N;
  FINISH(st);
}

int gcsph_update_rho(int64_t N, double* rho, const double* drho, double dt, double rho0, const int32_t* pt,
                     void* stream) {
  if (!rho || !drho || !pt) return fail(GCSPH_EINVAL, "null argument");
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  k_fn_update_rho<<<nblocks(N, PTPB), PTPB, 0, st>>>(N, rho, drho, dt, rho0, pt);
  FINISH(st);
}

int gcsph_update_v(int32_t D, int64_t N, double* const* v_dev, const double* const* a_dev, double dt,
                   const int32_t* pt, void* stream) {
  CHECK_D(D);
  W3 v;
  V3 a;
  int rc = vec_out(D, v_dev, &v, "v");
  if (!rc) rc = vec_in(D, a_dev, &a, "a");
  if (rc) return rc;
  if (!pt) return fail(GCSPH_EINVAL, "null ptype");
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DISPATCH(D, k_fn_update_v, nblocks(N, PTPB), st, N, v, a, dt, pt);
  FINISH(st);
}

int gcsph_update_x(int32_t D, int64_t N, double* const* x_dev, const double* const* v_dev, double dt, void* stream) {
  CHECK_D(D);
  W3 x;
  V3 v;
  int rc = vec_out(D, x_dev, &x, "x");
  if (!rc) rc = vec_in(D, v_dev, &v, "v");
  if (rc) return rc;
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DISPATCH(D, k_fn_update_x, nblocks(N, PTPB), st, N, x, v, dt);
  FINISH(st);
}

int gcsph_symplectic(int32_t D, int64_t N, double* rho, double* rhoh, double* const* v_dev, double* const* vh_dev,
                     double* const* x_dev, double* const* xh_dev, const double* drho, const double* const* a_dev,
                     double dt, double* const* cdx_dev, double rho0, const int32_t* pt, void* stream) {
  CHECK_D(D);
  W3 v, vh, x, xh, cdx;
  V3 a;
  int rc = vec_out(D, v_dev, &v, "v");
  if (!rc) rc = vec_out(D, vh_dev, &vh, "vh");
  if (!rc) rc = vec_out(D, x_dev, &x, "x");
  if (!rc) rc = vec_out(D, xh_dev, &xh, "xh");
  if (!rc) rc = vec_out(D, cdx_dev, &cdx, "cdx");
  if (!rc) rc = vec_in(D, a_dev, &a, "a");
  if (rc) return rc;
  if (!rho || !rhoh || !drho || !pt) return fail(GCSPH_EINVAL, "null argument");
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DISPATCH(D, k_fn_symplectic, nblocks(N, PTPB), st, N, rho, rhoh, v, vh, x, xh, drho, a, dt, cdx, rho0, pt);
  FINISH(st);
}

int gcsph_dpcreg(int32_t D, int64_t N, int64_t P, double* const* buf_dev, const double* const* v_dev,
                 const double* rho, const double* Pr, const int32_t* pairs, const double* const* x_dev, double l0,
                 double Pmin, double Pmax, double dt, double lambda, double kernlim, const int32_t* pt,
                 void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  W3 buf;
  V3 v, x;
  int rc = vec_out(D, buf_dev, &buf, "buf");
  if (!rc) rc = vec_in(D, v_dev, &v, "v");
  if (!rc) rc = vec_in(D, x_dev, &x, "x");
  if (rc) return rc;
  if (!rho || !Pr || !pt) return fail(GCSPH_EINVAL, "null argument");
  if (!(l0 > 0)) return fail(GCSPH_EINVAL, "l0 must be > 0");
  cudaStream_t st = (cudaStream_t)stream;
  for (int d = 0; d < D; ++d) GC_CUDA(cudaMemsetAsync(buf.p[d], 0, sizeof(double) * (size_t)N, st));
  double l0inv = 1.0 / l0;
  double nW = D == 2 ? wc2_norm_w<2>(l0inv) : wc2_norm_w<3>(l0inv);
  double whinv = 1.0 / wc2_w(0.5, nW);
  double eta2 = (0.1 * l0) * (0.1 * l0);
  if (P > 0) {
    DISPATCH(D, k_fn_dpc, nblocks(P, PTPB), st, P, buf, v, rho, Pr, pairs, x, l0inv, nW, whinv, Pmin, Pmax, dt,
             lambda, kernlim, eta2, pt);
    GC_LAUNCHED();
  }
  GC_CUDA(cudaStreamSynchronize(st));
  return GCSPH_OK;
}

int gcsph_update_dpcreg(int32_t D, int64_t N, double* const* v_dev, double* const* x_dev,
                        const double* const* buf_dev, double dt, const int32_t* pt, void* stream) {
  CHECK_D(D);
  W3 v, x;
  V3 buf;
  int rc = vec_out(D, v_dev, &v, "v");
  if (!rc) rc = vec_out(D, x_dev, &x, "x");
  if (!rc) rc = vec_in(D, buf_dev, &buf, "buf");
  if (rc) return rc;
  if (!pt) return fail(GCSPH_EINVAL, "null ptype");
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DISPATCH(D, k_fn_update_dpc, nblocks(N, PTPB), st, N, v, x, buf, dt, pt);
  FINISH(st);
}

int gcsph_xsphcorr(int32_t D, int64_t N, int64_t P, double* const* buf_dev, const int32_t* pairs, const double* W,
                   const double* rho, const double* const* v_dev, double m0, double eps, const int32_t* pt,
                   void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  W3 buf;
  V3 v;
  int rc = vec_out(D, buf_dev, &buf, "buf");
  if (!rc) rc = vec_in(D, v_dev, &v, "v");
  if (rc) return rc;
  if (!W || !rho || !pt) return fail(GCSPH_EINVAL, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  for (int d = 0; d < D; ++d) GC_CUDA(cudaMemsetAsync(buf.p[d], 0, sizeof(double) * (size_t)N, st));
  if (P > 0) {
    DISPATCH(D, k_fn_xsph, nblocks(P, PTPB), st, P, buf, pairs, W, rho, v, m0, eps, pt);
    GC_LAUNCHED();
  }
  GC_CUDA(cudaStreamSynchronize(st));
  return GCSPH_OK;
}

int gcsph_update_xsph(int32_t D, int64_t N, double* const* x_dev, const double* const* buf_dev, double dt,
                      const int32_t* pt, void* stream) {
  CHECK_D(D);
  W3 x;
  V3 buf;
  int rc = vec_out(D, x_dev, &x, "x");
  if (!rc) rc = vec_in(D, buf_dev, &buf, "buf");
  if (rc) return rc;
  if (!pt) return fail(GCSPH_EINVAL, "null ptype");
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  DISPATCH(D, k_fn_update_xsph, nblocks(N, PTPB), st, N, x, buf, dt, pt);
  FINISH(st);
}

int gcsph_cspmcorr(int32_t D, int64_t N, int64_t P, double* const* buf_dev, const double* W, double* rho, double m0,
                   const int32_t* pairs, const int32_t* pt, void* stream) {
  CHECK_D(D);
  CHECK_PAIRS(P, pairs);
  W3 buf;
  int rc = vec_out(D, buf_dev, &buf, "buf");
  if (rc) return rc;
  if (!W || !rho || !pt) return fail(GCSPH_EINVAL, "null argument");
  if (N <= 0) return GCSPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  for (int d = 0; d < D; ++d) GC_CUDA(cudaMemsetAsync(buf.p[d], 0, sizeof(double) * (size_t)N, st));
  if (P > 0) {
    k_fn_cspm1<<<nblocks(P, PTPB), PTPB, 0, st>>>(P, buf.p[0], buf.p[1], W, rho, m0, pairs, pt);
    GC_LAUNCHED();
  }
  k_fn_cspm2<<<nblocks(N, PTPB), PTPB, 0, st>>>(N, rho, buf.p[0], buf.p[1]);
  FINISH(st);
}

int gcsph_dt_stepping(int32_t D, int64_t N, const double* const* a_dev, const double* const* v_dev,
                      const double* const* x_dev, double c0, double h, double CFL, double tmin, double tmax,
                      double* dt_out, void* stream) {
  CHECK_D(D);
  V3 a, v, x;
  int rc = vec_in(D, a_dev, &a, "a");
  if (!rc) rc = vec_in(D, v_dev, &v, "v");
  if (!rc) rc = vec_in(D, x_dev, &x, "x");
  if (rc) return rc;
  if (!dt_out) return fail(GCSPH_EINVAL, "null dt_out");
  if (N <= 0) return fail(GCSPH_EINVAL, "empty problem");
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf tmp;
  if ((rc = tmp.ensure(2 * sizeof(unsigned long long), st, true))) return rc;
  double eta2 = (0.01 * h) * (0.01 * h);
  DISPATCH(D, k_fn_dt, nblocks(N, PTPB), st, N, a, v, x, h, eta2, tmp.as<unsigned long long>());
  GC_LAUNCHED();
  unsigned long long hb[2];
  cudaError_t e = cudaMemcpyAsync(hb, tmp.p, sizeof(hb), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  tmp.release();
  if (e != cudaSuccess) return cuda_fail(e, "dt readback", __FILE__, __LINE__);
  double amax, vmax;
  memcpy(&amax, &hb[0], 8);
  memcpy(&vmax, &hb[1], 8);
  double dt1 = sqrt(h / (3.0 * amax));
  double dt2 = h / (c0 + vmax);
  double dt = CFL * fmin(dt1, dt2);
  dt = fmin(fmax(dt, tmin), tmax);
  *dt_out = dt;
  return GCSPH_OK;
}

}  // extern "C"
