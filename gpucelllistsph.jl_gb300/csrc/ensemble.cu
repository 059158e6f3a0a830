// ensemble.cu -- batched FP32 SPH: many independent dam-break instances
// advanced together, one launch per pass over all of them.
//
// The reference steps one SPHProblem at a time (src/sphproblem.jl:204-345).
// Here every admitted instance lives in one segmented particle space:
// instance s owns particles [p_off_s, p_off_s + n_s) and cell keys
// [key_off_s, key_off_s + ncell_s), so one counting sort over the global keys
// keeps each instance's particles in its own range, in cell order, ties by
// the instance-local particle id (deterministic, and independent of which
// other instances are present).  The pair passes walk the 3^D neighbour cells
// of each particle directly (no neighbour list): the cell edge equals the
// kernel support H, so every pair within H is found, and every SPH term of the
// path vanishes beyond H.
//
// Precision: pair arithmetic and per-particle sums in FP32 (Kahan-compensated);
// density held as δρ = ρ - ρ₀ so the EOS (1+δρ/ρ₀)^γ - 1 and the
// density-diffusion difference (δρ_j - δρ_i) - ρ₀((1+ε)^(1/γ) - 1) carry no
// cancellation against ρ₀; positions in FP64 (the symplectic position update
// runs in FP64) and, for the pair passes, as FP32 offsets from the corner of
// the particle's cell, so a pair's separation is exact to ~1e-7 of H.
//
// Physics per pair and per particle follows the FP64 path kernel by kernel
// (∂ρ∂tDDT!, ∂v∂t!, ∂v∂t_av!, ∂v∂t_visc!, gravity!, fbmolforce!, ∂v∂tpF!,
// the half-step predictors and symplectic_update!), fixed Δt per instance.
#include <math.h>
#include <algorithm>
#include <map>
#include <vector>
#include "gcsph_common.cuh"

namespace gcsph {
namespace {

constexpr int ENS_MAX_TPB = 512;

// per-instance constants (device table, indexed by packing position)
struct EnsInst {
  // the stage passes' per-entry constants in 16-byte groups, so that a
  // branch loads the group it needs with one vector load
  float4 kA;      // H², 1/H, dwc, cell edge
  float4 kB;      // ρ₀, η², m₀, DDTgz
  float4 kC;      // kddt, kav, kvisc, (unused)
  float4 kD;      // pfcr, hp1, 2h, kpf
  float4 kE;      // pc[0..3]
  float4 kFB[2];  // fb_d, fb_r0, fb_eta2, (unused) of stage 1 and stage 2
  double origin[3];
  double csinv;  // 1 / cell edge
  double cs;
  double dt;
  int nc[3];
  int key_off;
  int gamma;
  int use_visc, use_pF;
  int cspmn;
  int use_dpc, use_xsph;
  float csf, H2, h, Hinv, nW, nDW, m0, rho0, c0, P0, alpha, DDTkh, DDTgz, eta2, g, nu, s, twoh, pfc, hp1;
  float fb_d[2], fb_r0[2], fb_eta2[2];  // fbmolforce constants of stage 1 and stage 2
  float pc[4];                           // (1+ε)^(1/γ) - 1 series coefficients
  float dpc_l0inv, dpc_nW, dpc_whinv, dpc_kernlim, dpc_eta2, dpc_pmin, dpc_pmax, dpc_lambda;
  float xsph_c;                          // 2 m0 ε
  float rho0inv, m0inv;                  // 1/ρ₀, 1/m₀
  float dwc;                             // -20 nDW / H: W'(r)/r = dwc (1 - r/H)^3
  float pfcr;                            // 1.5π / 2h: the cosine's argument per unit r in ∂v∂tpF!
  // products of the above that the stage passes use as one factor
  float kddt;                            // DDTkh m₀ (∂ρ∂tDDT!)
  float kav;                             // 2 α c₀ h m₀: ∂v∂t_av!'s -Π m₀ over (Δv·Δx) / ((r² + η²)(ρi + ρj))
  float kvisc;                           // 4 ν m₀ (∂v∂t_visc!)
  float kpf;                             // s / m₀ (∂v∂tpF!)
  int p_off;                             // first particle of the instance (list entries are instance-local)
  int reuse;                             // the list is kept while the particles stay within the skin
  float LR2;                             // list radius², (H (1 + skin))² = cell edge²
  float dthr2;                           // rebuild when a particle has moved more than about skin/2 (squared)
  float dpc_skip;                        // dpcreg! skips a row whose separations after the step stay above
                                         // this (l0 with a margin for FP32 rounding)
};

struct EnsArr {
  int64_t N;
  const int32_t* inst;
  const int32_t* skey;       // global cell key of each (sorted) particle
  const int32_t* cellstart;  // first particle of each global cell, K+1 entries
  double* x[3];              // positions (FP64)
  float* v[3];
  float* dr;                 // ρ - ρ₀
  float* drb;                // ρΔt½ - ρ₀ at the step's start: the predictor's base (cspmcorr! leaves it)
  const int32_t* pt;
  float* off[3];             // x - cell corner (FP32)
  float* offh[3];            // half-step positions - cell corner
  float* vh[3];               // also the dpcreg! sums, after the corrector
  float* drh;
  float* offn[3];            // x - cell corner after the corrector (dpcreg!)
  float* dxb[3];             // xΔt½ base - x: dpcreg!/xsphcorr! move x, not xΔt½
  float* dvb[3];             // vΔt½ base - v: dpcreg! moves v, not vΔt½
  int* nl;                   // neighbour list of the step, entry-major (q * ncap + i); written with
                             // streaming stores (evict-first in L2)
  int* nlc;                  // entries per particle
  int64_t ncap;              // particle capacity (the list's row pitch)
  int nls;                   // entries per particle the list holds
  int* ovf;                  // a row outgrew nls: every later kernel of the call skips
  int* nlmax;                // the longest row seen (to size the next try)
  // packed per-particle records that neighbours read (float4 loads):
  //   r1 (2 float4): x offset, v, δρ, ptype       -- stage 1, the list build
  //   r2 (2 or 3):   xΔt½ offset, vΔt½, δρΔt½, ptype, x offset -- stage 2
  float4* r1;
  float4* r2;
  // records of the correction passes, in r1's layout (offsets, v, δρ, ptype):
  //   r3: offsets after the corrector -- dpcreg!'s neighbours (null: no DPC)
  //   r4: offsets at the step's start, v after dpcreg! -- xsphcorr!, cspmcorr!
  //       and dpcreg!'s pair test (null: none of the three)
  float4* r3;
  float4* r4;
  const int32_t* istep;      // steps done per instance (cspmcorr! schedule)
  const int* rb;             // per instance: this step rebuilds the instance's cells and list
  float* ob[3];              // offsets at the instance's last list build (same cell corner as off)
  // dpcreg!'s row bound (null: every row is scanned): the smallest r² of each
  // row at the step's start (stage 1) and, per instance, the largest |Δx|² of
  // the step (after the corrector)
  float* rmin2;
  const unsigned* sdmax;
};

// record layouts (D = 2 | D = 3); P = the EOS of the record's density, where
// a slot is free, so that neighbours read it instead of evaluating it
//   r1: [o0 o1 v0 v1][dr pt P -]        | [o0 o1 o2 v0][v1 v2 dr pt]
//   r2: [h0 h1 w0 w1][drh pt o0 o1]     | [h0 h1 h2 w0][w1 w2 drh pt][o0 o1 o2 P]
template <int D, int S>
__host__ __device__ constexpr bool rec_has_p() {
  return (D == 2 && S == 1) || (D == 3 && S == 2);
}
template <int D>
__device__ __forceinline__ void put_r1(float4* r, int64_t k, const float* o, const float* v, float dr, int pt,
                                       float P) {
  if (D == 2) {
    r[2 * k] = make_float4(o[0], o[1], v[0], v[1]);
    r[2 * k + 1] = make_float4(dr, __int_as_float(pt), P, 0.f);
  } else {
    r[2 * k] = make_float4(o[0], o[1], o[D - 1], v[0]);
    r[2 * k + 1] = make_float4(v[1], v[D - 1], dr, __int_as_float(pt));
  }
}
// raw record of neighbour j for stage S (2 float4, or 3 for stage 2 in 3-D)
template <int D, int S>
struct Rec {
  float4 a, b, c;
};
template <int D, int S>
__device__ __forceinline__ Rec<D, S> load_rec(const float4* __restrict__ r1, const float4* __restrict__ r2, int j) {
  Rec<D, S> x;
  if (S == 1) {
    x.a = __ldg(r1 + 2 * (int64_t)j);
    x.b = __ldg(r1 + 2 * (int64_t)j + 1);
  } else if (D == 2) {
    x.a = __ldg(r2 + 2 * (int64_t)j);
    x.b = __ldg(r2 + 2 * (int64_t)j + 1);
  } else {
    x.a = __ldg(r2 + 3 * (int64_t)j);
    x.b = __ldg(r2 + 3 * (int64_t)j + 1);
    x.c = __ldg(r2 + 3 * (int64_t)j + 2);
  }
  return x;
}
// decode: o = offset at x, h = offset at xΔt½ (stage 2), v, δρ, ptype, and
// P where the record holds it (rec_has_p)
template <int D, int S>
__device__ __forceinline__ void decode_rec(const Rec<D, S>& x, float* o, float* h, float* v, float& dr, int& pt,
                                           float& P) {
  if (S == 1) {
    if (D == 2) {
      o[0] = x.a.x; o[1] = x.a.y; v[0] = x.a.z; v[1] = x.a.w;
      dr = x.b.x; pt = __float_as_int(x.b.y); P = x.b.z;
    } else {
      o[0] = x.a.x; o[1] = x.a.y; o[D - 1] = x.a.z; v[0] = x.a.w;
      v[1] = x.b.x; v[D - 1] = x.b.y; dr = x.b.z; pt = __float_as_int(x.b.w);
    }
  } else {
    if (D == 2) {
      h[0] = x.a.x; h[1] = x.a.y; v[0] = x.a.z; v[1] = x.a.w;
      dr = x.b.x; pt = __float_as_int(x.b.y); o[0] = x.b.z; o[1] = x.b.w;
    } else {
      h[0] = x.a.x; h[1] = x.a.y; h[D - 1] = x.a.z; v[0] = x.a.w;
      v[1] = x.b.x; v[D - 1] = x.b.y; dr = x.b.z; pt = __float_as_int(x.b.w);
      o[0] = x.c.x; o[1] = x.c.y; o[D - 1] = x.c.z; P = x.c.w;
    }
  }
}

template <int D>
__device__ __forceinline__ void put_r2(float4* r, int64_t k, const float* h, const float* w, float drh, int pt,
                                       const float* o, float P) {
  if (D == 2) {
    r[2 * k] = make_float4(h[0], h[1], w[0], w[1]);
    r[2 * k + 1] = make_float4(drh, __int_as_float(pt), o[0], o[1]);
  } else {
    r[3 * k] = make_float4(h[0], h[1], h[D - 1], w[0]);
    r[3 * k + 1] = make_float4(w[1], w[D - 1], drh, __int_as_float(pt));
    r[3 * k + 2] = make_float4(o[0], o[1], o[D - 1], P);
  }
}

struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// Kahan sums of the x and y components in packed FP32 pairs (sm_100's
// two-wide FADD/FFMA): the compensation is kept negated, nc = -c, so that
// every step is an add or a fused multiply-add by -1 -- y = x + nc,
// t = s + y, nc = (s - t) + y -- bit for bit the scalar KSum on each lane
struct KSum2 {
  float2 s = make_float2(0.f, 0.f), nc = make_float2(0.f, 0.f);
  __device__ __forceinline__ void add(float2 x) {
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 y = __fadd2_rn(x, nc);
    const float2 t = __fadd2_rn(s, y);
    nc = __fadd2_rn(__ffma2_rn(t, m1, s), y);
    s = t;
  }
  __device__ __forceinline__ KSum part(int q) const {
    KSum k;
    k.s = q == 0 ? s.x : s.y;
    k.c = q == 0 ? -nc.x : -nc.y;
    return k;
  }
};

// √x for x >= 0 by the approximate reciprocal root (within a few ulp); 0 at 0
__device__ __forceinline__ float sqrt_fast(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }

template <int D>
__device__ __forceinline__ float dot32(const float* a, const float* b) {
  float r = a[0] * b[0];
#pragma unroll
  for (int d = 1; d < D; ++d) r = fmaf(a[d], b[d], r);
  return r;
}

// P0 ((1+e)^γ - 1), e = δρ/ρ₀, without cancellation (pressure(), src/gpukernels_sph.jl:691-697)
__device__ __forceinline__ float eos32(float dr, int pt, const EnsInst& I) {
  if (pt <= 1 && dr < 0.f) return 0.f;
  const float e = dr * I.rho0inv;
  float p;
  if (I.gamma == 7)
    p = e * (7.f + e * (21.f + e * (35.f + e * (35.f + e * (21.f + e * (7.f + e))))));
  else
    p = expm1f((float)I.gamma * log1pf(e));
  return I.P0 * p;
}


// (1+ε)^(1/γ) - 1 (powfancy7th(1+ε) - 1, src/gpukernels_sph.jl:499-515), from
// the series coefficients pc
__device__ __forceinline__ float root_m1g(float eps, const float4& pc, int gamma) {
  if (fabsf(eps) < 0.01f) return eps * (pc.x + eps * (pc.y + eps * (pc.z + eps * pc.w)));
  return powf(1.f + eps, 1.f / (float)gamma) - 1.f;
}

__device__ __forceinline__ void cell_of(int key, const EnsInst& I, int& c0, int& c1, int& c2) {
  int local = key - I.key_off;
  c0 = local % I.nc[0];
  local /= I.nc[0];
  c1 = local % I.nc[1];
  c2 = local / I.nc[1];
}

// ---------------------------------------------------------------------------
// binning (segmented counting sort)
// ---------------------------------------------------------------------------
// An instance that keeps its list keeps its particles' cells (the key they
// were sorted by, skey): the sort then leaves its particles where they are,
// so the list's instance-local indices stay valid.
template <int D>
__global__ void k_ens_key(int64_t N, const int32_t* __restrict__ inst, const double* __restrict__ x0,
                          const double* __restrict__ x1, const double* __restrict__ x2,
                          const EnsInst* __restrict__ T, const int* __restrict__ rb,
                          const int32_t* __restrict__ skey, int32_t* __restrict__ key, int32_t* __restrict__ slot,
                          int32_t* __restrict__ count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int si = inst[i];
  int k;
  if (!rb[si]) {
    k = skey[i];
  } else {
    const EnsInst& I = T[si];
    const double xs[3] = {x0[i], x1[i], D == 3 ? x2[i] : 0.0};
    int c[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double f = floor((xs[d] - I.origin[d]) * I.csinv);
      f = f >= 0.0 ? f : 0.0;  // also NaN -> 0: points outside the frozen grid clamp to its edge cells
      c[d] = f < (double)(I.nc[d] - 1) ? (int)f : I.nc[d] - 1;
    }
    k = I.key_off + c[0] + I.nc[0] * (c[1] + I.nc[1] * c[2]);
  }
  key[i] = k;
  slot[i] = atomicAdd(&count[k], 1);
}

__global__ void k_ens_scatter(int64_t N, const int32_t* __restrict__ key, const int32_t* __restrict__ slot,
                              const int32_t* __restrict__ cellstart, int32_t* __restrict__ tmp) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  tmp[cellstart[key[i]] + slot[i]] = (int32_t)i;
}

// rank inside the cell by instance-local id (ids are unique inside an instance)
__global__ void k_ens_rank(int64_t N, const int32_t* __restrict__ tmp, const int32_t* __restrict__ key,
                           const int32_t* __restrict__ cellstart, const int32_t* __restrict__ id,
                           int32_t* __restrict__ perm) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= N) return;
  const int32_t i = tmp[q];
  const int32_t c = key[i];
  const int32_t s = cellstart[c], e = cellstart[c + 1];
  const int32_t oi = id[i];
  int32_t r = 0;
  for (int32_t t = s; t < e; ++t) r += id[tmp[t]] < oi;
  perm[s + r] = i;
}

struct EnsState {
  double* x[3];
  float* v[3];
  float* dxb[3];
  float* dvb[3];
  float* dr;
  float* drb;
  int32_t* pt;
  int32_t* id;
};

// new[k] = old[perm[k]]; FP32 offsets from the new cell's corner
template <int D>
__global__ void k_ens_permute(int64_t N, const int32_t* __restrict__ perm, const int32_t* __restrict__ key,
                              const int32_t* __restrict__ inst, const EnsInst* __restrict__ T, EnsState in,
                              EnsState out, int32_t* __restrict__ skey, float* __restrict__ o0,
                              float* __restrict__ o1, float* __restrict__ o2, float4* __restrict__ r1,
                              const int* __restrict__ rb, float* __restrict__ b0, float* __restrict__ b1,
                              float* __restrict__ b2) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  const int32_t i = perm[k];
  const int32_t kk = key[i];
  skey[k] = kk;
  const bool reb = rb[inst[k]] != 0;
  const EnsInst& I = T[inst[k]];
  int c0, c1, c2;
  cell_of(kk, I, c0, c1, c2);
  float ov[D], vv[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double xv = in.x[d][i];
    out.x[d][k] = xv;
    vv[d] = in.v[d][i];
    out.v[d][k] = vv[d];
    out.dxb[d][k] = in.dxb[d][i];
    out.dvb[d][k] = in.dvb[d][i];
    const int cd = d == 0 ? c0 : (d == 1 ? c1 : c2);
    float* o = d == 0 ? o0 : (d == 1 ? o1 : o2);
    ov[d] = (float)(xv - (I.origin[d] + (double)cd * I.cs));
    o[k] = ov[d];
    if (reb) (d == 0 ? b0 : (d == 1 ? b1 : b2))[k] = ov[d];
  }
  const float dr = in.dr[i];
  const int pt = in.pt[i];
  out.dr[k] = dr;
  out.drb[k] = in.drb[i];
  out.pt[k] = pt;
  out.id[k] = in.id[i];
  put_r1<D>(r1, k, ov, vv, dr, pt, D == 2 ? eos32(dr, pt, I) : 0.f);
}

// ---------------------------------------------------------------------------
// neighbour list, built after the re-sort of the instances that rebuild: the
// 3^D cell walk with the pair test r < H (1 + skin) at x (FP32 offsets).  An
// entry is the neighbour's instance-local index above 6 bits of cell shift,
// (dx+1) | (dy+1) << 2 | (dz+1) << 4 (the index is below 2^26, so the entry
// is read as unsigned).  Every pass keeps only the entries with r < H at the
// step's x, so the pairs of a step are those the reference's update! finds,
// whichever step built the list.  Stored entry-major (entry q of particle i
// at q*ncap + i) so that the passes' loads coalesce.  A row that outgrows the
// stride raises *ovf: every later kernel of the call skips, the host grows
// the stride and repeats.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int ent_code(int dxc, int dy, int dz) {
  return (dxc + 1) | ((dy + 1) << 2) | ((dz + 1) << 4);
}
__device__ __forceinline__ int ent_make(int j_local, int code) { return (int)(((unsigned)j_local << 6) | code); }
__device__ __forceinline__ int ent_index(int ent) { return (int)((unsigned)ent >> 6); }

// An entry's cell shift per axis, field - 1 in {-1, 0, 1}, as floats.  Each
// 2-bit field is OR-ed into the low mantissa bits of 1.5 * 2^23
// (0x4B400000), where it reads as 12582912 + field exactly, and one
// subtraction leaves field - 1; the separation then takes the shift times
// the cell edge in one fused multiply-add.
template <int D>
__device__ __forceinline__ void ent_shift(int ent, float* s) {
  const unsigned u = (unsigned)ent;
  s[0] = __uint_as_float((u & 3u) | 0x4B400000u) - 12582913.f;
  s[1] = __uint_as_float(((u >> 2) & 3u) | 0x4B400000u) - 12582913.f;
  if (D == 3) s[D - 1] = __uint_as_float(((u >> 4) & 3u) | 0x4B400000u) - 12582913.f;
}

// a candidate's decision: with L lanes on a particle, a ballot keeps the hits
// in candidate order, so the list is the same for every L
template <int L>
__device__ __forceinline__ void nl_emit(const EnsArr& A, int64_t i, int lane, unsigned gm, unsigned gbase, bool hit,
                                        int j, int code, int& cnt) {
  if (L == 1) {
    if (hit) {
      if (cnt < A.nls) __stcs(A.nl + (int64_t)cnt * A.ncap + i, ent_make(j, code));
      ++cnt;
    }
  } else {
    const unsigned bal = (__ballot_sync(gm, hit) >> gbase) & (L == 32 ? 0xffffffffu : ((1u << L) - 1u));
    const int at = cnt + __popc(bal & ((1u << lane) - 1u));
    if (hit && at < A.nls) __stcs(A.nl + (int64_t)at * A.ncap + i, ent_make(j, code));
    cnt += __popc(bal);
  }
}

__device__ __forceinline__ void nl_close(const EnsArr& A, int64_t i, int lane, int cnt) {
  if (lane == 0) {
    A.nlc[i] = cnt < A.nls ? cnt : A.nls;
    if (cnt > A.nls) {
      atomicMax(A.nlmax, cnt);
      *A.ovf = 1;
    }
  }
}

// L lanes share a particle: candidates go in chunks of L
template <int D, int L>
__global__ void __launch_bounds__(ENS_MAX_TPB) k_ens_nlist(EnsArr A, const EnsInst* __restrict__ T) {
  if (*A.ovf) return;
  const unsigned lanew = threadIdx.x & 31u;
  const unsigned gbase = lanew & ~(unsigned)(L - 1);
  const unsigned gm = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << gbase);
  const int lane = (int)(lanew - gbase);
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / L;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / L; i < A.N; i += groups) {
    if (!A.rb[A.inst[i]]) continue;  // the instance keeps its list
    const EnsInst& I = T[A.inst[i]];
    int cx0, cy0, cz0;
    cell_of(A.skey[i], I, cx0, cy0, cz0);
    float oi[D];
#pragma unroll
    for (int d = 0; d < D; ++d) oi[d] = A.off[d][i];
    int cnt = 0;
    const int zlo = D == 3 ? -1 : 0, zhi = D == 3 ? 1 : 0;
    for (int dz = zlo; dz <= zhi; ++dz) {
      const int cz = cz0 + dz;
      if (cz < 0 || cz >= I.nc[2]) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        const int cy = cy0 + dy;
        if (cy < 0 || cy >= I.nc[1]) continue;
        const int row = I.key_off + I.nc[0] * (cy + I.nc[1] * cz);
        for (int dxc = -1; dxc <= 1; ++dxc) {
          const int cx = cx0 + dxc;
          if (cx < 0 || cx >= I.nc[0]) continue;
          const int j0 = A.cellstart[row + cx], j1 = A.cellstart[row + cx + 1];
          const float shx = (float)dxc * I.csf, shy = (float)dy * I.csf, shz = (float)dz * I.csf;
          const int code = ent_code(dxc, dy, dz);
          for (int jb = j0; jb < j1; jb += L) {
            const int j = jb + lane;
            bool hit = false;
            if (j < j1 && j != i) {
              float d[D];
#pragma unroll
              for (int q = 0; q < D; ++q) d[q] = (oi[q] - A.off[q][j]) - (q == 0 ? shx : (q == 1 ? shy : shz));
              hit = dot32<D>(d, d) < I.LR2;
            }
            nl_emit<L>(A, i, lane, gm, gbase, hit, j - I.p_off, code, cnt);
          }
        }
      }
    }
    nl_close(A, i, lane, cnt);
  }
}

// ---------------------------------------------------------------------------
// Tiled list build: a block takes a tile of up to `cpb` consecutive cells of
// one x-row of one instance.  In the sorted particle order the tile's 3^D
// neighbourhood is 3^(D-1) contiguous particle ranges, one per (dy, dz) row
// (cells cx0-1 .. cx1), so the block stages their FP32 offsets in shared
// memory with coalesced copies (cp.async) and runs the candidate loop of
// k_ens_nlist out of shared memory: the same candidates in the same order
// through the same ballot, so the list is the same for every variant.  With
// staging depth 2 the next tile's ranges are copied while the current tile is
// tested.  A tile whose neighbourhood does not fit the buffer reads global
// memory instead.  Tiles are numbered instance by instance (tile_off: the
// first tile of each instance, in packing order), row by row, along x.
// ---------------------------------------------------------------------------
constexpr int TILE_CPB_MAX = 16;
constexpr int TILE_TPB = 128;

__device__ __forceinline__ void cp_async4(void* dst_smem, const void* src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

struct TileSm {
  int s, cxa, rowkey;           // instance, first staged cell, key of cell 0 of the home row
  int hs, he, total, staged;    // home particles [hs, he), staged particle count, fits the buffer
  int rok[9];                   // the (dy, dz) row lies inside the grid
  int delta[9];                 // buffer index - particle index, per row
  int cs[9][TILE_CPB_MAX + 3];  // cell starts (particle indices) of cells cxa .. cxb + 1, per row
};

// the geometry of tile t, by warp 0
template <int D>
__device__ void tile_geometry(const EnsArr& A, const EnsInst* __restrict__ T, const int* __restrict__ tile_off,
                              int ninst, int cpb, int cap, int t, TileSm& G) {
  constexpr int NR = D == 3 ? 9 : 3;
  const int lane = threadIdx.x & 31;
  int s = 0;
  if (lane == 0) {
    int lo = 0, hi = ninst;  // tile_off[lo] <= t < tile_off[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (tile_off[mid] <= t)
        lo = mid;
      else
        hi = mid;
    }
    s = lo;
  }
  s = __shfl_sync(0xffffffffu, s, 0);
  const EnsInst& I = T[s];
  const int tpr = (I.nc[0] + cpb - 1) / cpb;
  const int lt = t - tile_off[s];
  const int row = lt / tpr;
  const int cx0 = (lt - row * tpr) * cpb;
  const int cx1 = min(cx0 + cpb, I.nc[0]);
  const int cy = row % I.nc[1], cz = row / I.nc[1];
  const int cxa = max(cx0 - 1, 0), cxb = min(cx1, I.nc[0] - 1);
  const int ncs = cxb - cxa + 2;
  for (int q = lane; q < NR * ncs; q += 32) {
    const int r = q / ncs, c = q - r * ncs;
    const int y = cy + (r % 3) - 1, z = cz + (D == 3 ? r / 3 - 1 : 0);
    const bool in = y >= 0 && y < I.nc[1] && z >= 0 && z < I.nc[2];
    G.cs[r][c] = in ? A.cellstart[I.key_off + cxa + c + I.nc[0] * (y + I.nc[1] * z)] : 0;
  }
  __syncwarp();
  if (lane == 0) {
    int tot = 0;
    for (int r = 0; r < NR; ++r) {
      const int y = cy + (r % 3) - 1, z = cz + (D == 3 ? r / 3 - 1 : 0);
      const bool in = y >= 0 && y < I.nc[1] && z >= 0 && z < I.nc[2];
      G.rok[r] = in;
      G.delta[r] = tot - G.cs[r][0];
      tot += in ? G.cs[r][ncs - 1] - G.cs[r][0] : 0;
    }
    constexpr int CR = D == 3 ? 4 : 1;  // the home row (dy = dz = 0)
    G.s = s;
    G.cxa = cxa;
    G.rowkey = I.key_off + I.nc[0] * (cy + I.nc[1] * cz);
    G.hs = G.cs[CR][cx0 - cxa];
    G.he = A.rb[s] ? G.cs[CR][cx1 - cxa] : G.hs;  // an instance that keeps its list: nothing to do
    G.total = tot;
    G.staged = tot <= cap;
  }
}

// copies of the tile's staged offsets (every thread; cp.async, not waited on)
template <int D>
__device__ __forceinline__ void tile_stage(const EnsArr& A, const TileSm& G, float* buf, int cap) {
  constexpr int NR = D == 3 ? 9 : 3;
  if (!G.staged || G.hs == G.he) return;  // no home particles: nothing to test
  for (int q = threadIdx.x; q < G.total; q += blockDim.x) {
    // row r fills buffer indices [delta[r] + cs[r][0], delta[r + 1] + cs[r + 1][0])
    int r = 0;
    while (r < NR - 1 && q >= G.delta[r + 1] + G.cs[r + 1][0]) ++r;
    const int j = q - G.delta[r];
#pragma unroll
    for (int d = 0; d < D; ++d) cp_async4(buf + d * cap + q, A.off[d] + j);
  }
}

// the home particles of one tile: k_ens_nlist's loop, offsets from the buffer
template <int D, int L, bool STAGED>
__device__ __forceinline__ void tile_particles(const EnsArr& A, const EnsInst& I, const TileSm& G,
                                               const float* __restrict__ buf, int cap) {
  constexpr int NR = D == 3 ? 9 : 3;
  constexpr int CR = D == 3 ? 4 : 1;
  const unsigned lanew = threadIdx.x & 31u;
  const unsigned gbase = lanew & ~(unsigned)(L - 1);
  const unsigned gm = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << gbase);
  const int lane = (int)(lanew - gbase);
  const int groups = blockDim.x / L;
  for (int i = G.hs + (int)threadIdx.x / L; i < G.he; i += groups) {
    const int cxi = A.skey[i] - G.rowkey;
    float oi[D];
#pragma unroll
    for (int d = 0; d < D; ++d) oi[d] = STAGED ? buf[d * cap + i + G.delta[CR]] : A.off[d][i];
    int cnt = 0;
    for (int r = 0; r < NR; ++r) {
      if (!G.rok[r]) continue;
      const int dy = r % 3 - 1, dz = D == 3 ? r / 3 - 1 : 0;
      const int dl = G.delta[r];
      for (int dxc = -1; dxc <= 1; ++dxc) {
        const int cx = cxi + dxc;
        if (cx < 0 || cx >= I.nc[0]) continue;
        const int lc = cx - G.cxa;
        const int j0 = G.cs[r][lc], j1 = G.cs[r][lc + 1];
        const float shx = (float)dxc * I.csf, shy = (float)dy * I.csf, shz = (float)dz * I.csf;
        const int code = ent_code(dxc, dy, dz);
        for (int jb = j0; jb < j1; jb += L) {
          const int j = jb + lane;
          bool hit = false;
          if (j < j1 && j != i) {
            float d[D];
#pragma unroll
            for (int q = 0; q < D; ++q)
              d[q] = (oi[q] - (STAGED ? buf[q * cap + j + dl] : A.off[q][j])) - (q == 0 ? shx : (q == 1 ? shy : shz));
            hit = dot32<D>(d, d) < I.LR2;
          }
          nl_emit<L>(A, i, lane, gm, gbase, hit, j - I.p_off, code, cnt);
        }
      }
    }
    nl_close(A, i, lane, cnt);
  }
}

template <int D, int L, int DEPTH>
__global__ void __launch_bounds__(TILE_TPB) k_ens_nlist_tile(EnsArr A, const EnsInst* __restrict__ T,
                                                             const int* __restrict__ tile_off, int ninst, int cpb,
                                                             int cap) {
  if (*A.ovf) return;
  extern __shared__ float4 tile_smem[];
  float* const sbuf = reinterpret_cast<float*>(tile_smem);
  __shared__ TileSm G[DEPTH];
  const int ntiles = tile_off[ninst];
  const bool w0 = threadIdx.x < 32;
  int t = blockIdx.x;
  if (t >= ntiles) return;
  int cur = 0;
  if (w0) tile_geometry<D>(A, T, tile_off, ninst, cpb, cap, t, G[0]);
  __syncthreads();
  tile_stage<D>(A, G[0], sbuf, cap);
  cp_async_commit();
  for (;;) {
    const int nt = t + gridDim.x;
    if (DEPTH == 2) {
      // the next tile's copies go out before this tile is tested
      const int nx = cur ^ 1;
      if (nt < ntiles) {
        if (w0) tile_geometry<D>(A, T, tile_off, ninst, cpb, cap, nt, G[nx]);
        __syncthreads();
        tile_stage<D>(A, G[nx], sbuf + nx * D * cap, cap);
      }
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const TileSm& g = G[cur];
    if (g.staged)
      tile_particles<D, L, true>(A, T[g.s], g, sbuf + cur * D * cap, cap);
    else
      tile_particles<D, L, false>(A, T[g.s], g, nullptr, cap);
    if (nt >= ntiles) break;
    __syncthreads();  // the buffer and geometry just used are refilled next
    if (DEPTH == 2) {
      cur ^= 1;
    } else {
      if (w0) tile_geometry<D>(A, T, tile_off, ninst, cpb, cap, nt, G[0]);
      __syncthreads();
      tile_stage<D>(A, G[0], sbuf, cap);
      cp_async_commit();
    }
    t = nt;
  }
}

// ---------------------------------------------------------------------------
// the two pair passes over the step's neighbour list, persistent grid-stride
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool cspm_due(const EnsInst& I, const int32_t* istep, int s) {
  return I.cspmn > 0 && (istep[s] + 1) % I.cspmn == 0;
}

// lanes per particle in the pair passes: fixed per dimension (never tuned),
// so that the summation order -- and every result -- is the same whatever
// the launch shape and whatever else is in the ensemble
// (measured on GB300: 2 in 2-D beats 1 and 4; 4 in 3-D beats 2 and 8)
template <int D>
__host__ __device__ constexpr int stage_lanes() {
  return D == 2 ? 2 : 4;
}

// Kahan partial sums of the L lanes of a particle, combined by a fixed butterfly
template <int L>
__device__ __forceinline__ float lane_total(const KSum& k, unsigned gm) {
  float s = k.s, c = k.c;
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) {
    s += __shfl_xor_sync(gm, s, o);
    c += __shfl_xor_sync(gm, c, o);
  }
  return s - c;
}

// two blocks of 512 per SM: at most 64 registers.  RM (stage 1): keep each
// row's smallest r² for dpcreg!'s row bound (a separate instantiation, so the
// ensembles without dpcreg! run the loop without it)
template <int D, int STAGE, bool RM = false>
__global__ void __launch_bounds__(ENS_MAX_TPB, 2) k_ens_stage(EnsArr A, const EnsInst* __restrict__ T) {
  if (*A.ovf) return;
  constexpr int L = stage_lanes<D>();
  const unsigned lanew = threadIdx.x & 31u;
  const unsigned gbase = lanew & ~(unsigned)(L - 1);
  const unsigned gm = ((1u << L) - 1u) << gbase;
  const int lane = (int)(lanew - gbase);
  const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / L;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / L; i < A.N; i += groups) {
    const EnsInst& I = T[A.inst[i]];
    float oi[D], ohi[D], vi[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      oi[d] = A.off[d][i];
      ohi[d] = STAGE == 1 ? oi[d] : A.offh[d][i];
      vi[d] = STAGE == 1 ? A.v[d][i] : A.vh[d][i];
    }
    const int pti = A.pt[i];
    const float dri = STAGE == 1 ? A.dr[i] : A.drh[i];
    const float rhoi = I.rho0 + dri;
    const float irhoi = __fdividef(1.f, rhoi);
    const float Pi = eos32(dri, pti, I);
    const int fbs = STAGE - 1;
    KSum drho;
    KSum2 accxy;  // the x and y components of the acceleration, packed
    KSum accz;
    float rm2 = INFINITY;  // stage 1: the row's smallest r² (dpcreg!'s row bound)
    const int nn = A.nlc[i];
    // the next entry is loaded one iteration ahead: the list streams from
    // DRAM, and its latency then overlaps the current neighbour's arithmetic
    int nxt = lane < nn ? A.nl[(int64_t)lane * A.ncap + i] : 0;
    for (int e = lane; e < nn; e += L) {
      const int ent = nxt;
      if (e + L < nn) nxt = A.nl[(int64_t)(e + L) * A.ncap + i];
      const Rec<D, STAGE> rec = load_rec<D, STAGE>(A.r1, A.r2, I.p_off + ent_index(ent));
      float sh[D];
      ent_shift<D>(ent, sh);
      // the neighbour's record: offsets (at x, and at xΔt½ in stage 2), velocity, δρ, ptype
      float oj[D], hj[D], vj[D], drj, Prec = 0.f;
      int ptj;
      decode_rec<D, STAGE>(rec, oj, hj, vj, drj, ptj, Prec);
      const float4 kA = I.kA;  // H², 1/H, dwc, cell edge
      float d[D];
#pragma unroll
      for (int q = 0; q < D; ++q) d[q] = fmaf(-sh[q], kA.w, oi[q] - oj[q]);
      const float r2 = dot32<D>(d, d);
      if (STAGE == 1 && RM) rm2 = fminf(rm2, r2);
      if (!(r2 < kA.x)) continue;  // in the list's skin: not a pair of this step
      // sph∇W!: W'(r)/r of WendlandC2 = -20 nDW Hinv (1-q)^3.  Reciprocals and
      // roots here are the approximate intrinsics (within 2 ulp each), far
      // inside the FP32 path's error against FP64.
      const float r = r2 > 0.f ? r2 * rsqrtf(r2) : 0.f;
      const float u = r * kA.y;
      const float t = u < 1.f ? 1.f - u : 0.f;
      const float dwr = kA.z * (t * t * t);
      float gw[D], dd[D], dv[D];
#pragma unroll
      for (int q = 0; q < D; ++q) {
        gw[q] = d[q] * dwr;
        dd[q] = STAGE == 1 ? d[q] : fmaf(-sh[q], kA.w, ohi[q] - hj[q]);
        dv[q] = vi[q] - vj[q];
      }
      const float4 kB = I.kB;  // ρ₀, η², m₀, DDTgz
      const float r2d = STAGE == 1 ? r2 : dot32<D>(dd, dd);
      const float rhoj = kB.x + drj;
      const float irhoj = __fdividef(1.f, rhoj);
      const bool both = pti > 0 && ptj > 0;
      const float inv = __fdividef(1.f, r2d + kB.y);
      // gsc: the factor of ∇W of ∂v∂t! and ∂v∂t_av! together; f: the
      // viscous, surface-tension and boundary terms
      float gsc = 0.f, f[D];
#pragma unroll
      for (int q = 0; q < D; ++q) f[q] = 0.f;
      if (pti * ptj > 0) {
        // ∂v∂t!
        float Pj = Prec;
        if (!rec_has_p<D, STAGE>()) Pj = eos32(drj, ptj, I);
        gsc = -kB.z * (Pi + Pj) * (irhoi * irhoj);
      }
      if (both) {
        const float4 kC = I.kC;  // kddt, kav, kvisc
        const float ddgw = dot32<D>(dd, gw);
        // ∂ρ∂tDDT!
        float term = kB.z * dot32<D>(dv, gw);
        if (pti > 1) {
          const float dp = kB.x * root_m1g(kB.w * dd[1], I.kE, I.gamma);
          term += kC.x * ((drj - dri) - dp) * inv * (-ddgw) * irhoj;
        }
        drho.add(term);
        const float cond = dot32<D>(dv, dd);
        if (cond < 0.f || I.use_visc) {
          const float ii = __fdividef(1.f, rhoi + rhoj) * inv;
          // ∂v∂t_av!: -Π m₀ = 2 α c₀ h m₀ (Δv·Δx) / ((r² + η²)(ρi + ρj))
          if (cond < 0.f) gsc += kC.y * cond * ii;
          if (I.use_visc) {
            // ∂v∂t_visc!
            const float nt = kC.z * ddgw * ii;
#pragma unroll
            for (int q = 0; q < D; ++q) f[q] = nt * dv[q];
          }
        }
        if (I.use_pF) {
          // ∂v∂tpF! (in stage 1 the separation is r itself)
          const float4 kD = I.kD;  // pfcr, hp1, 2h, kpf
          const float rd = STAGE == 1 ? r : (r2d > 0.f ? r2d * rsqrtf(r2d) : 0.f);
          if (rd < kD.z) {
            const float scos = kD.w * __cosf(kD.x * rd) * __fdividef(1.f, rd + kD.y);  // argument in [0, 1.5π)
#pragma unroll
            for (int q = 0; q < D; ++q) f[q] = fmaf(scos, dd[q], f[q]);
          }
        }
      }
      if ((pti > 0) != (ptj > 0)) {
        const float4 kF = I.kFB[fbs];  // fb_d, fb_r0, fb_eta2
        if (r < kF.y) {
          // fbmolforce! at x
          const float qq = kF.y * __fdividef(1.f, r + kF.z);
          const float q2 = qq * qq, q4 = q2 * q2, q8 = q4 * q4;
          const float Fc = kF.x * (q8 * q4 - q4) * __fdividef(1.f, r2 + kF.z);
#pragma unroll
          for (int q = 0; q < D; ++q) f[q] += d[q] * Fc;
        }
      }
      accxy.add(make_float2(fmaf(gsc, gw[0], f[0]), fmaf(gsc, gw[1], f[1])));
      if (D == 3) accz.add(fmaf(gsc, gw[D - 1], f[D - 1]));
    }
    KSum acc[D];
    acc[0] = accxy.part(0);
    acc[1] = accxy.part(1);
    if (D == 3) acc[D - 1] = accz;
    float a[D];
#pragma unroll
    for (int q = 0; q < D; ++q) a[q] = lane_total<L>(acc[q], gm) - (q == 1 ? I.g : 0.f);
    const float drho_s = lane_total<L>(drho, gm);
    if (STAGE == 1 && RM) {
#pragma unroll
      for (int o = L / 2; o > 0; o >>= 1) rm2 = fminf(rm2, __shfl_xor_sync(gm, rm2, o));
    }
    if (lane != 0) continue;
    if (STAGE == 1 && RM) A.rmin2[i] = rm2;
    const float dt = (float)I.dt;
    if (STAGE == 1) {
      // update_ρp∂ρ∂tΔt!, update_vp∂v∂tΔt!, update_xpvΔt! at Δt/2
      const float hdt = 0.5f * dt;
      float drh = A.drb[i] + drho_s * hdt;
      if (drh < 0.f && pti < 0) drh = 0.f;
      A.drh[i] = drh;
      float hh[D], ww[D];
#pragma unroll
      for (int q = 0; q < D; ++q) {
        float vh = vi[q] + A.dvb[q][i];
        if (pti > 1) vh = vh + a[q] * hdt;
        A.vh[q][i] = vh;
        ww[q] = vh;
        hh[q] = (oi[q] + A.dxb[q][i]) + vh * hdt;
        A.offh[q][i] = hh[q];
      }
      put_r2<D>(A.r2, i, hh, ww, drh, pti, oi, D == 3 ? eos32(drh, pti, I) : 0.f);
    } else {
      // symplectic_update!: δρ_new = δρ - ρ 2ε/(2+ε), positions in FP64
      const float dr0 = A.dr[i];
      const float epsi = -(drho_s / rhoi) * dt;
      float dn = dr0 - (I.rho0 + dr0) * (2.f * epsi / (2.f + epsi));
      if (dn < 0.f && pti <= 1) dn = 0.f;
      A.dr[i] = dn;
      A.drb[i] = dn;
      float nvs[D], ons[D];
#pragma unroll
      for (int q = 0; q < D; ++q) {
        const float v0 = A.v[q][i];
        const float nv = pti > 1 ? v0 + a[q] * dt : v0;
        A.v[q][i] = nv;
        nvs[q] = nv;
        const double ddx = ((double)v0 + (double)nv) * 0.5 * I.dt;
        A.x[q][i] = A.x[q][i] + ddx;
        ons[q] = oi[q] + (float)ddx;
        A.offn[q][i] = ons[q];
        A.dxb[q][i] = 0.f;
        A.dvb[q][i] = 0.f;
      }
      if (A.r3 && I.use_dpc) put_r1<D>(A.r3, i, ons, nvs, dn, pti, 0.f);
      if (A.r4 && (I.use_dpc || I.use_xsph || cspm_due(I, A.istep, A.inst[i])))
        put_r1<D>(A.r4, i, oi, nvs, dn, pti, 0.f);
    }
  }
}

// dpcreg! (src/gpukernels_sph.jl:1500-1553) at the corrected state: pairs of
// the step (at x), terms at x_{n+1}, v_{n+1}, ρ_{n+1} and P(ρ_{n+1}); the sums
// go to the vΔt½ buffer (free after the corrector) and k_ens_dpc_apply runs
// update_dpcreg! (:1617-1632)
template <int D>
__global__ void __launch_bounds__(ENS_MAX_TPB) k_ens_dpc(EnsArr A, const EnsInst* __restrict__ T) {
  if (*A.ovf) return;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.N; i += stride) {
    const EnsInst& I = T[A.inst[i]];
    if (!I.use_dpc) continue;
    const int pti = A.pt[i];
    KSum sum[D];
    if (pti > 0) {
      float ni[D], vi[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        ni[d] = A.offn[d][i];
        vi[d] = A.v[d][i];
      }
      // the row bound: a pair is within l0 after the step only if its
      // separation at the step's start, less both particles' moves, is; the
      // row's smallest separation, its own move and the instance's largest
      // move clear l0 for every entry, so every term would be skipped below
      bool scan = true;
      if (A.rmin2) {
        float di2 = 0.f;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          const float dd = ni[d] - A.off[d][i];
          di2 = fmaf(dd, dd, di2);
        }
        const float lo = sqrtf(A.rmin2[i]) - sqrtf(di2) - sqrtf(__uint_as_float(A.sdmax[A.inst[i]]));
        scan = !(lo >= I.dpc_skip);
      }
      const float dri = A.dr[i];
      const float rhoi = I.rho0 + dri, Pi = eos32(dri, pti, I);
      const float dt = (float)I.dt;
      const int nn = scan ? A.nlc[i] : 0;
      int nxt = nn > 0 ? A.nl[i] : 0;  // entries one iteration ahead (as in the stage passes)
      for (int e = 0; e < nn; ++e) {
        const int ent = nxt;
        if (e + 1 < nn) nxt = A.nl[(int64_t)(e + 1) * A.ncap + i];
        const int j = I.p_off + ent_index(ent);
        // the neighbour after the corrector: its record's first half holds
        // the offsets; beyond l0 (u >= 1) W, χ and Pᵇ vanish and so does the
        // pair's dpcreg! term, so the rest is read only within l0
        const float4 ra = __ldg(A.r3 + 2 * (int64_t)j);
        float sh[D];
        ent_shift<D>(ent, sh);
        const float onj[3] = {ra.x, ra.y, D == 3 ? ra.z : 0.f};
        float dx[D];
#pragma unroll
        for (int q = 0; q < D; ++q) dx[q] = fmaf(-sh[q], I.csf, ni[q] - onj[q]);
        const float r2 = dot32<D>(dx, dx);
        const float u = sqrt_fast(r2) * I.dpc_l0inv;
        if (!(u < 1.f)) continue;
        const float4 rb = __ldg(A.r3 + 2 * (int64_t)j + 1);
        const float vj[3] = {D == 2 ? ra.z : ra.w, D == 2 ? ra.w : rb.x, D == 2 ? 0.f : rb.y};
        const float drj = D == 2 ? rb.x : rb.z;
        const int ptj = __float_as_int(D == 2 ? rb.y : rb.w);
        if (!(ptj > 0)) continue;
        if (I.reuse) {
          // a pair of this step: r < H at the step's starting positions
          const float4 sj = __ldg(A.r4 + 2 * (int64_t)j);
          const float oj[3] = {sj.x, sj.y, sj.z};
          float dm[D];
#pragma unroll
          for (int q = 0; q < D; ++q) dm[q] = fmaf(-sh[q], I.csf, A.off[q][i] - oj[q]);
          if (!(dot32<D>(dm, dm) < I.H2)) continue;
        }
        float dv[D];
#pragma unroll
        for (int q = 0; q < D; ++q) dv[q] = vi[q] - vj[q];
        const float rhoj = I.rho0 + drj;
        const float t = 1.f - u;
        const float t2 = t * t;
        const float w = (1.f + 4.f * u) * (t2 * t2) * I.dpc_nW;
        const float chi = sqrt_fast(w * I.dpc_whinv);
        const float kk = u < I.dpc_kernlim ? 1.f : chi;
        const float Pb = chi * fmaxf(fminf(I.dpc_lambda * fabsf(Pi + eos32(drj, ptj, I)),
                                           I.dpc_lambda * I.dpc_pmax), I.dpc_pmin);
        const float vr = dot32<D>(dv, dx);
        float c;
        if (vr < 0.f) c = kk * (-vr * __fdividef(1.f, r2 + I.dpc_eta2));
        else c = 2.f * dt * Pb * __fdividef(1.f, (rhoi + rhoj) * (r2 + I.dpc_eta2));
#pragma unroll
        for (int q = 0; q < D; ++q) sum[q].add(c * dx[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < D; ++q) A.vh[q][i] = sum[q].s;
  }
}

template <int D>
__global__ void k_ens_dpc_apply(EnsArr A, const EnsInst* __restrict__ T) {
  if (*A.ovf) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.N) return;
  const EnsInst& I = T[A.inst[i]];
  if (!I.use_dpc || !(A.pt[i] > 1)) return;
  float nv[D], o[D];
#pragma unroll
  for (int q = 0; q < D; ++q) {
    const float s = A.vh[q][i];
    nv[q] = A.v[q][i] + s;
    A.v[q][i] = nv[q];
    A.dvb[q][i] -= s;
    const double dx = (double)s * I.dt;
    A.x[q][i] = A.x[q][i] + dx;
    A.offn[q][i] += (float)dx;
    A.dxb[q][i] -= (float)dx;
    o[q] = A.off[q][i];
  }
  put_r1<D>(A.r4, i, o, nv, A.dr[i], A.pt[i], 0.f);  // the later passes see v after dpcreg!
}

// xsphcorr! + update_xsphcorr! (src/gpukernels_sph.jl:1745-1838): stage-1 W
// (pairs and distances at x), v and ρ after the corrector and dpcreg!;
// moves x only.  Reads neighbours' v, writes its own x: one pass.  Little
// arithmetic per neighbour and a record gather each: latency-bound, so three
// blocks of 512 per SM (at most 42 registers) rather than the stage passes' two
template <int D>
__global__ void __launch_bounds__(ENS_MAX_TPB, 3) k_ens_xsph(EnsArr A, const EnsInst* __restrict__ T) {
  if (*A.ovf) return;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.N; i += stride) {
    const EnsInst& I = T[A.inst[i]];
    if (!I.use_xsph || !(A.pt[i] > 1)) continue;
    float oi[D], vi[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      oi[d] = A.off[d][i];
      vi[d] = A.v[d][i];
    }
    const float rhoi = I.rho0 + A.dr[i];
    KSum sum[D];
    const int nn = A.nlc[i];
    int nxt = nn > 0 ? A.nl[i] : 0;  // entries one iteration ahead (as in the stage passes)
    for (int e = 0; e < nn; ++e) {
      const int ent = nxt;
      if (e + 1 < nn) nxt = A.nl[(int64_t)(e + 1) * A.ncap + i];
      const int j = I.p_off + ent_index(ent);
      float oj[D], hj[D], vj[D], drj, pu;
      int ptj;
      decode_rec<D, 1>(load_rec<D, 1>(A.r4, nullptr, j), oj, hj, vj, drj, ptj, pu);
      if (!(ptj > 1)) continue;
      float sh[D];
      ent_shift<D>(ent, sh);
      float d[D];
#pragma unroll
      for (int q = 0; q < D; ++q) d[q] = fmaf(-sh[q], I.csf, oi[q] - oj[q]);
      const float r2 = dot32<D>(d, d);
      if (!(r2 < I.H2)) continue;  // in the list's skin
      const float u = sqrt_fast(r2) * I.Hinv;
      const float t = u < 1.f ? 1.f - u : 0.f;
      const float t2 = t * t;
      const float w = (1.f + 4.f * u) * (t2 * t2) * I.nW;
      const float xs = I.xsph_c * w * __fdividef(1.f, rhoi + (I.rho0 + drj));
#pragma unroll
      for (int q = 0; q < D; ++q) sum[q].add((vj[q] - vi[q]) * xs);
    }
#pragma unroll
    for (int q = 0; q < D; ++q) {
      const double dx = (double)sum[q].s * I.dt;
      A.x[q][i] = A.x[q][i] + dx;
      A.offn[q][i] += (float)dx;
      A.dxb[q][i] -= (float)dx;
    }
  }
}

// cspmcorr! (src/gpukernels_sph.jl:1693-1719) of the instances whose step
// count reaches a multiple of cspmn with this step: ρ = Σ m0 W / Σ (m0/ρ_j) W
// over real neighbours at the step's starting positions, with the updated ρ_j;
// formed as δρ = Σ m0 W δρ_j/ρ_j / Σ m0 W/ρ_j (no cancellation against ρ₀).
// The result goes to δρ½ (free after the corrector) and is applied by
// k_ens_cspm_apply, so every particle reads the pre-correction densities.

template <int D>
__global__ void __launch_bounds__(ENS_MAX_TPB) k_ens_cspm(EnsArr A, const EnsInst* __restrict__ T,
                                                          const int32_t* __restrict__ istep) {
  if (*A.ovf) return;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < A.N; i += stride) {
    const int s = A.inst[i];
    const EnsInst& I = T[s];
    if (!cspm_due(I, istep, s)) continue;
    const float dri = A.dr[i];
    if (!(A.pt[i] > 0)) {
      A.drh[i] = dri;  // Σ over nothing: 0/0, the reference keeps ρ
      continue;
    }
    float oi[D];
#pragma unroll
    for (int d = 0; d < D; ++d) oi[d] = A.off[d][i];
    KSum s2, s3;
    const int nn = A.nlc[i];
    int nxt = nn > 0 ? A.nl[i] : 0;  // entries one iteration ahead (as in the stage passes)
    for (int e = 0; e < nn; ++e) {
      const int ent = nxt;
      if (e + 1 < nn) nxt = A.nl[(int64_t)(e + 1) * A.ncap + i];
      const int j = I.p_off + ent_index(ent);
      float oj[D], hj[D], vj[D], drj, pu;
      int ptj;
      decode_rec<D, 1>(load_rec<D, 1>(A.r4, nullptr, j), oj, hj, vj, drj, ptj, pu);
      if (!(ptj > 0)) continue;
      float sh[D];
      ent_shift<D>(ent, sh);
      float d[D];
#pragma unroll
      for (int q = 0; q < D; ++q) d[q] = fmaf(-sh[q], I.csf, oi[q] - oj[q]);
      const float r2 = dot32<D>(d, d);
      if (!(r2 < I.H2)) continue;  // in the list's skin
      const float u = sqrt_fast(r2) * I.Hinv;
      const float t = u < 1.f ? 1.f - u : 0.f;
      const float t2 = t * t;
      const float w = (1.f + 4.f * u) * (t2 * t2) * I.nW;
      const float mw = I.m0 * w * __fdividef(1.f, I.rho0 + drj);
      s2.add(mw);
      s3.add(mw * drj);
    }
    const float nd = s3.s / s2.s;
    A.drh[i] = nd == nd ? nd : dri;
  }
}

__global__ void k_ens_cspm_apply(int64_t N, const int32_t* __restrict__ inst, const EnsInst* __restrict__ T,
                                 const int32_t* __restrict__ istep, const float* __restrict__ drh,
                                 float* __restrict__ dr, const int* __restrict__ ovf) {
  if (*ovf) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int s = inst[i];
  if (cspm_due(T[s], istep, s)) dr[i] = drh[i];
}

// the largest squared displacement since the last list build, per instance
// (particles are sorted by instance: a warp's lanes of one instance reduce
// together, one atomic per instance per warp)
// STEP: the largest move of the step (x_{n+1} - x_n, after the corrector) of
// the instances with dpcreg!, for its row bound; NaN gives +inf (no row skips)
template <int D, bool STEP>
__global__ void k_ens_disp(EnsArr A, const EnsInst* __restrict__ T, unsigned* __restrict__ dmax) {
  if (*A.ovf) return;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = i < A.N;
  const int s = in ? A.inst[i] : -1;
  unsigned bits = 0u;
  if (in && (STEP ? T[s].use_dpc : T[s].reuse)) {
    float d2 = 0.f;
#pragma unroll
    for (int q = 0; q < D; ++q) {
      const float dd = A.offn[q][i] - (STEP ? A.off[q][i] : A.ob[q][i]);
      d2 = fmaf(dd, dd, d2);
    }
    bits = d2 == d2 ? __float_as_uint(d2) : 0x7f800000u;  // NaN: rebuild
  }
  // the common case: the block's particles belong to one instance -- one
  // atomic per block (per-warp atomics on a few hundred addresses contend)
  __shared__ int s_first;
  __shared__ unsigned s_wmax[32];
  if (threadIdx.x == 0) s_first = s;
  __syncthreads();
  if (__syncthreads_and(s == s_first)) {
    const unsigned m = __reduce_max_sync(0xffffffffu, bits);
    if ((threadIdx.x & 31) == 0) s_wmax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned b = 0u;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b = max(b, s_wmax[w]);
      if (in && b != 0u) atomicMax(dmax + s, b);
    }
    return;
  }
  const unsigned grp = __match_any_sync(0xffffffffu, s);
  const unsigned m = __reduce_max_sync(grp, bits);
  if (in && m != 0u && (threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(dmax + s, m);
}

// one more step done, per instance, and for the call; whether the instance
// rebuilds its list at the next step (always without a skin)
__global__ void k_ens_tick(int ninst, int32_t* __restrict__ istep, const int* __restrict__ ovf,
                           int* __restrict__ done, const EnsInst* __restrict__ T, int* __restrict__ rb,
                           int* __restrict__ nreb, unsigned* __restrict__ dmax, unsigned* __restrict__ sdmax) {
  if (*ovf) return;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < ninst) {
    istep[s] += 1;
    if (rb[s]) nreb[s] += 1;
    rb[s] = T[s].reuse ? (__uint_as_float(dmax[s]) > T[s].dthr2 ? 1 : 0) : 1;
    dmax[s] = 0u;
    sdmax[s] = 0u;
  }
  if (s == 0) *done += 1;
}

// gather one instance's field into its original particle order
__global__ void k_ens_out(int64_t n, int64_t p0, const int32_t* __restrict__ id, const double* __restrict__ xd,
                          const float* __restrict__ xf, const int32_t* __restrict__ xi, int mode, double base,
                          double* __restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t q = p0 + k;
  double v;
  if (mode == 0) v = xd[q];
  else if (mode == 1) v = base + (double)xf[q];
  else v = (double)xi[q];
  out[id[q]] = v;
}

__global__ void k_ens_pressure_out(int64_t n, int64_t p0, const int32_t* __restrict__ id,
                                   const float* __restrict__ dr, const int32_t* __restrict__ pt,
                                   const EnsInst* __restrict__ T, int si, double* __restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t q = p0 + k;
  out[id[q]] = (double)eos32(dr[q], pt[q], T[si]);
}

__global__ void k_fill_i32(int32_t* __restrict__ p, int64_t n, int32_t v) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) p[k] = v;
}

// repack after a removal: new range r takes old particles [old_off, old_off + n)
struct Move {
  int64_t new_off, old_off, n;
};
__global__ void k_ens_repack(int nmoves, const Move* __restrict__ mv, int64_t N, int D, EnsState in, EnsState out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  int lo = 0, hi = nmoves - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mv[mid].new_off <= k) lo = mid;
    else hi = mid - 1;
  }
  const int64_t src = mv[lo].old_off + (k - mv[lo].new_off);
  for (int d = 0; d < D; ++d) {
    out.x[d][k] = in.x[d][src];
    out.v[d][k] = in.v[d][src];
    out.dxb[d][k] = in.dxb[d][src];
    out.dvb[d][k] = in.dvb[d][src];
  }
  out.dr[k] = in.dr[src];
  out.drb[k] = in.drb[src];
  out.pt[k] = in.pt[src];
  out.id[k] = in.id[src];
}

// the same repack for one 32-bit per-particle array (out must not alias in)
__global__ void k_ens_repack32(int nmoves, const Move* __restrict__ mv, int64_t N, const int32_t* __restrict__ in,
                               int32_t* __restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  int lo = 0, hi = nmoves - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mv[mid].new_off <= k) lo = mid;
    else hi = mid - 1;
  }
  out[k] = in[mv[lo].old_off + (k - mv[lo].new_off)];
}

// cell keys follow their instance's new key offset after a removal
__global__ void k_ens_shift_keys(int64_t N, const int32_t* __restrict__ inst, const int32_t* __restrict__ delta,
                                 int32_t* __restrict__ skey) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N) return;
  skey[k] += delta[inst[k]];
}

}  // namespace
}  // namespace gcsph

using namespace gcsph;

struct EnsHostInst {
  int32_t slot;
  int64_t n, p_off;
  int64_t filled_off = -1;  // p_off the per-particle instance index was last written for
  int64_t filled_idx = -1;
  int64_t key_off, ncell;
  gcsph_ens_params prm;
  int64_t steps;
  int rb = 1;        // rebuilds its list at its next step (mirrors the device flag across layout changes)
  int32_t nreb = 0;  // list builds so far
  EnsInst dev;
};

struct EnsGraph {
  int64_t n_steps = -1, N = -1, K = -1, gen = -1;
  int cur = -1, tpb = 0, timing = 0, nl_lanes = 0, nl_cpb = -1, nl_depth = 0, nl_cap = 0, dpc_bound = -1;
  cudaGraphExec_t exec = nullptr;
  unsigned long long used = 0;
  long long launches = 0;
  std::vector<TimerRec> timers;
};

struct gcsph_ens {
  int D = 2;
  cudaStream_t st = 0;
  cudaStream_t cap = nullptr;
  std::vector<EnsHostInst> inst;  // packing order
  int32_t next_slot = 0;
  int64_t N = 0, K = 0, cap_n = 0, cap_k = 0;
  int cur = 0;
  int64_t gen = 0;  // layout generation (graphs and tuning follow it)
  // state, double-buffered for the re-sort
  DevBuf X[2][3], V[2][3], DXB[2][3], DVB[2][3], DR[2], DRB[2], PT[2], ID[2];
  DevBuf OFFN[3];
  DevBuf INST, KEY, SLOT, TMP, PERM, SKEY, OFF[3], OFFH[3], VH[3], DRH, COUNT, CELLSTART, SCRATCH, TAB, MOVES, OUT;
  DevBuf ISTEP;          // steps done per instance (cspmcorr! schedule), packing order
  DevBuf NL, NLC;        // neighbour list of the step and its row lengths
  DevBuf FLAGS;          // [0] list overflow, [1] longest row, [2] steps done in the call
  DevBuf R1, R2;         // packed neighbour records of the two stages
  DevBuf R3, R4;         // packed neighbour records of the correction passes
  DevBuf OB[3];          // offsets at each instance's last list build
  DevBuf RB, NREB, DMAX; // per instance: rebuild at the next step, list builds, largest displacement²
  DevBuf SDMAX;          // per instance: largest |Δx|² of the step (dpcreg!'s row bound)
  DevBuf RMIN;           // per particle: smallest r² of the row at the step's start (dpcreg!'s row bound)
  bool dpc_bound = true; // dpcreg! skips the rows the bound clears (the results are the same)
  double skin = 0.05;    // list radius H (1 + skin); 0: every step rebuilds
  bool lists_lost = false;  // the list buffer was dropped: every instance rebuilds
  int nls = 0;           // list entries per particle (grows on overflow)
  int64_t nl_cap = 0;    // particles the list is sized for
  int tpb = 0;           // 0: not tuned yet
  bool tpb_fixed = false;
  int64_t tuned_n = 0;   // particle count the choice was made on
  int sms = 0, occ[4] = {0, 0, 0, 0}, occ_nl[4] = {0, 0, 0, 0}, occ_x[4] = {0, 0, 0, 0};
  int nl_lanes = 4;      // lanes per particle in the list build (tuned after the block size)
  int nl_cpb = 0;        // list build: 0 = a thread group per particle, else tiles of nl_cpb cells per block
  int nl_depth = 1;      // tiles staged ahead (1 or 2)
  int nl_cap_fix = 0;    // staged particles per tile buffer (0: from the lattice estimate)
  bool nl_fixed = false; // list build set by the caller: not tuned
  int tune_phase = 0;    // tuning done so far: 1 block size, 2 list lanes, 3 list tiles
  double ppc = 1.0;      // particles per cell estimate, (H / dx)^D over the instances
  DevBuf TILES;          // first tile of each instance, one table per cells-per-block choice
  int ntiles[4] = {0, 0, 0, 0};
  EnsGraph graphs[4];
  unsigned long long clock = 0;
  bool use_graphs = true;
  bool any_cspm = false;  // some instance runs cspmcorr!
  bool any_dpc = false, any_xsph = false;
  int64_t n_captures = 0, n_replays = 0;
};

namespace {

const int kTpbs[3] = {128, 256, 512};
const int kCpbs[4] = {2, 4, 8, 16};  // cells-per-block choices of the tiled list build

int cpb_index(int cpb) {
  for (int t = 0; t < 4; ++t)
    if (kCpbs[t] == cpb) return t;
  return -1;
}

// staged particles a tile buffer holds: the lattice estimate of the
// neighbourhood with a margin, within 96 KB of shared memory per block
int tile_cap(const gcsph_ens* e, int cpb, int depth) {
  const int per = depth * e->D * (int)sizeof(float);
  const int hi = (96 * 1024) / per / 32 * 32;
  if (e->nl_cap_fix > 0) return std::min(e->nl_cap_fix, hi);
  const double rows = e->D == 3 ? 9.0 : 3.0;
  const double want = 1.25 * (cpb + 2) * rows * e->ppc + 32.0;
  int cap = (int)std::min<double>(want, (double)hi);
  cap = (cap + 31) / 32 * 32;
  return std::max(32, std::min(cap, hi));
}

EnsState ens_state(gcsph_ens* e, int b) {
  EnsState s{};
  for (int d = 0; d < 3; ++d) {
    s.x[d] = e->X[b][d].as<double>();
    s.v[d] = e->V[b][d].as<float>();
    s.dxb[d] = e->DXB[b][d].as<float>();
    s.dvb[d] = e->DVB[b][d].as<float>();
  }
  s.dr = e->DR[b].as<float>();
  s.drb = e->DRB[b].as<float>();
  s.pt = e->PT[b].as<int32_t>();
  s.id = e->ID[b].as<int32_t>();
  return s;
}

EnsArr ens_arr(gcsph_ens* e) {
  EnsArr A{};
  A.N = e->N;
  A.inst = e->INST.as<int32_t>();
  A.skey = e->SKEY.as<int32_t>();
  A.cellstart = e->CELLSTART.as<int32_t>();
  for (int d = 0; d < 3; ++d) {
    A.x[d] = e->X[e->cur][d].as<double>();
    A.v[d] = e->V[e->cur][d].as<float>();
    A.off[d] = e->OFF[d].as<float>();
    A.offh[d] = e->OFFH[d].as<float>();
    A.vh[d] = e->VH[d].as<float>();
    A.offn[d] = e->OFFN[d].as<float>();
    A.dxb[d] = e->DXB[e->cur][d].as<float>();
    A.dvb[d] = e->DVB[e->cur][d].as<float>();
  }
  A.dr = e->DR[e->cur].as<float>();
  A.drb = e->DRB[e->cur].as<float>();
  A.drh = e->DRH.as<float>();
  A.nl = e->NL.as<int>();
  A.nlc = e->NLC.as<int>();
  A.ncap = e->nl_cap;
  A.nls = e->nls;
  A.ovf = e->FLAGS.as<int>();
  A.nlmax = e->FLAGS.as<int>() + 1;
  A.r1 = e->R1.as<float4>();
  A.r2 = e->R2.as<float4>();
  A.pt = e->PT[e->cur].as<int32_t>();
  A.rb = e->RB.as<int>();
  A.r3 = e->any_dpc ? e->R3.as<float4>() : nullptr;
  A.r4 = (e->any_dpc || e->any_xsph || e->any_cspm) ? e->R4.as<float4>() : nullptr;
  A.istep = e->ISTEP.as<int32_t>();
  for (int d = 0; d < 3; ++d) A.ob[d] = e->OB[d < e->D ? d : 0].as<float>();
  A.rmin2 = (e->any_dpc && e->dpc_bound) ? e->RMIN.as<float>() : nullptr;
  A.sdmax = e->SDMAX.as<unsigned>();
  return A;
}

void graph_free(EnsGraph& g) {
  if (g.exec) cudaGraphExecDestroy(g.exec);
  timer_release(g.timers);
  g = EnsGraph{};
}

void graphs_free(gcsph_ens* e) {
  for (EnsGraph& g : e->graphs) graph_free(g);
}

// grow every per-particle buffer to hold n particles (keeps the first N)
int ens_reserve(gcsph_ens* e, int64_t n) {
  if (n <= e->cap_n) return GCSPH_OK;
  const int64_t want = std::max<int64_t>(n, e->cap_n + e->cap_n / 2 + 1024);
  // move live state through fresh buffers: DevBuf::ensure does not keep contents
  int rc;
  for (int b = 0; b < 2; ++b) {
    auto keep = [&](DevBuf& buf, size_t esz) -> int {
      DevBuf fresh;
      int r = fresh.ensure(esz * want, e->st);
      if (r) return r;
      if (b == e->cur && e->N > 0 && buf.p)
        GC_CUDA(cudaMemcpyAsync(fresh.p, buf.p, esz * e->N, cudaMemcpyDeviceToDevice, e->st));
      GC_CUDA(cudaStreamSynchronize(e->st));
      buf.release();
      buf = fresh;
      fresh.p = nullptr;
      return GCSPH_OK;
    };
    for (int d = 0; d < e->D; ++d) {
      if ((rc = keep(e->X[b][d], sizeof(double)))) return rc;
      if ((rc = keep(e->V[b][d], sizeof(float)))) return rc;
      if ((rc = keep(e->DXB[b][d], sizeof(float)))) return rc;
      if ((rc = keep(e->DVB[b][d], sizeof(float)))) return rc;
    }
    if ((rc = keep(e->DR[b], sizeof(float)))) return rc;
    if ((rc = keep(e->DRB[b], sizeof(float)))) return rc;
    if ((rc = keep(e->PT[b], sizeof(int32_t)))) return rc;
    if ((rc = keep(e->ID[b], sizeof(int32_t)))) return rc;
  }
  DevBuf* i32[] = {&e->INST, &e->KEY, &e->SLOT, &e->TMP, &e->PERM};
  for (DevBuf* b : i32)
    if ((rc = b->ensure(sizeof(int32_t) * want, e->st))) return rc;
  // kept across the growth: the cells and build offsets of instances that keep their lists
  auto keep1 = [&](DevBuf& buf, size_t esz) -> int {
    DevBuf fresh;
    int r = fresh.ensure(esz * want, e->st);
    if (r) return r;
    if (e->N > 0 && buf.p) GC_CUDA(cudaMemcpyAsync(fresh.p, buf.p, esz * e->N, cudaMemcpyDeviceToDevice, e->st));
    GC_CUDA(cudaStreamSynchronize(e->st));
    buf.release();
    buf = fresh;
    fresh.p = nullptr;
    return GCSPH_OK;
  };
  if ((rc = keep1(e->SKEY, sizeof(int32_t)))) return rc;
  for (int d = 0; d < e->D; ++d)
    if ((rc = keep1(e->OB[d], sizeof(float)))) return rc;
  for (EnsHostInst& h : e->inst) h.filled_off = -1;  // the instance index buffer was reallocated
  for (int d = 0; d < e->D; ++d) {
    if ((rc = e->OFF[d].ensure(sizeof(float) * want, e->st))) return rc;
    if ((rc = e->OFFH[d].ensure(sizeof(float) * want, e->st))) return rc;
    if ((rc = e->VH[d].ensure(sizeof(float) * want, e->st))) return rc;
    if ((rc = e->OFFN[d].ensure(sizeof(float) * want, e->st))) return rc;
  }
  if ((rc = e->DRH.ensure(sizeof(float) * want, e->st))) return rc;
  if ((rc = e->RMIN.ensure(sizeof(float) * want, e->st))) return rc;
  if ((rc = e->R1.ensure(sizeof(float4) * 2 * want, e->st))) return rc;
  if ((rc = e->R2.ensure(sizeof(float4) * (e->D == 2 ? 2 : 3) * want, e->st))) return rc;
  if ((rc = e->R3.ensure(sizeof(float4) * 2 * want, e->st))) return rc;
  if ((rc = e->R4.ensure(sizeof(float4) * 2 * want, e->st))) return rc;
  if ((rc = e->SCRATCH.ensure(sizeof(int64_t) * scan_scratch_elems(std::max<int64_t>(want, e->cap_k) + 1), e->st)))
    return rc;
  e->cap_n = want;
  return GCSPH_OK;
}

int ens_reserve_cells(gcsph_ens* e, int64_t k) {
  if (k + 1 > (int64_t)INT32_MAX) return fail(GCSPH_ECAPACITY, "ensemble cell count past 2^31");
  if (k <= e->cap_k) return GCSPH_OK;
  const int64_t want = std::max<int64_t>(k, e->cap_k + e->cap_k / 2 + 4096);
  int rc;
  if ((rc = e->COUNT.ensure(sizeof(int32_t) * want, e->st))) return rc;
  if ((rc = e->CELLSTART.ensure(sizeof(int32_t) * (want + 1), e->st))) return rc;
  if ((rc = e->SCRATCH.ensure(sizeof(int64_t) * scan_scratch_elems(std::max<int64_t>(want, e->cap_n) + 1), e->st)))
    return rc;
  e->cap_k = want;
  return GCSPH_OK;
}

// the step's neighbour list: nls entries for each of cap_n particles
int ens_reserve_list(gcsph_ens* e, int nls) {
  if (nls <= e->nls && e->nl_cap >= e->cap_n) return GCSPH_OK;
  const int want = std::max(nls, e->nls);
  if ((double)want * (double)e->cap_n * 4.0 > 64e9) return fail(GCSPH_ENOMEM, "neighbour list too large");
  int rc;
  // the rows of instances that keep their lists move to the new buffer
  DevBuf nl, nlc;
  if ((rc = nl.ensure(sizeof(int) * (size_t)want * (size_t)e->cap_n, e->st))) return rc;
  if ((rc = nlc.ensure(sizeof(int) * (size_t)e->cap_n, e->st))) {
    nl.release();
    return rc;
  }
  // (rows past the old pitch belong to instances added since, which build theirs)
  const int64_t rows = std::min<int64_t>(e->N, e->nl_cap);
  if (e->NL.p && e->NLC.p && e->nls > 0 && rows > 0) {
    GC_CUDA(cudaMemcpy2DAsync(nl.p, sizeof(int) * (size_t)e->cap_n, e->NL.p, sizeof(int) * (size_t)e->nl_cap,
                              sizeof(int) * (size_t)rows, (size_t)e->nls, cudaMemcpyDeviceToDevice, e->st));
    GC_CUDA(cudaMemcpyAsync(nlc.p, e->NLC.p, sizeof(int) * (size_t)rows, cudaMemcpyDeviceToDevice, e->st));
  } else {
    e->lists_lost = true;
  }
  GC_CUDA(cudaStreamSynchronize(e->st));
  e->NL.release();
  e->NLC.release();
  e->NL = nl;
  e->NLC = nlc;
  nl.p = nlc.p = nullptr;
  if ((rc = e->FLAGS.ensure(sizeof(int) * 4, e->st, true))) return rc;
  e->nls = want;
  e->nl_cap = e->cap_n;
  e->gen += 1;  // captured graphs point at the old list
  graphs_free(e);
  return GCSPH_OK;
}

// the device's per-instance list flags into the host records (before a layout change)
int ens_pull_flags(gcsph_ens* e) {
  const size_t ni = e->inst.size();
  if (ni == 0 || !e->RB.p || !e->NREB.p) return GCSPH_OK;
  std::vector<int32_t> rb(ni), nreb(ni);
  GC_CUDA(cudaMemcpyAsync(rb.data(), e->RB.p, sizeof(int32_t) * ni, cudaMemcpyDeviceToHost, e->st));
  GC_CUDA(cudaMemcpyAsync(nreb.data(), e->NREB.p, sizeof(int32_t) * ni, cudaMemcpyDeviceToHost, e->st));
  GC_CUDA(cudaStreamSynchronize(e->st));
  for (size_t si = 0; si < ni; ++si) {
    e->inst[si].rb = e->lists_lost ? 1 : rb[si];
    e->inst[si].nreb = nreb[si];
  }
  return GCSPH_OK;
}

// device instance table + per-particle instance index after a layout change
int ens_relayout(gcsph_ens* e) {
  int64_t p = 0, k = 0;
  for (EnsHostInst& h : e->inst) {
    h.p_off = p;
    h.dev.p_off = (int)p;
    h.key_off = k;
    h.dev.key_off = (int)k;
    p += h.n;
    k += h.ncell;
  }
  if (p >= (int64_t)1 << 26) return fail(GCSPH_ECAPACITY, "ensemble of %lld particles: at most 2^26", (long long)p);
  e->N = p;
  e->K = k;
  e->any_cspm = e->any_dpc = e->any_xsph = false;
  for (const EnsHostInst& h : e->inst) {
    e->any_cspm = e->any_cspm || h.prm.cspmn > 0;
    e->any_dpc = e->any_dpc || h.prm.dpc_l0 > 0;
    e->any_xsph = e->any_xsph || h.prm.xsph_eps > 0;
  }
  int rc;
  if ((rc = ens_reserve_cells(e, k))) return rc;
  std::vector<EnsInst> tab(e->inst.size());
  for (size_t s = 0; s < e->inst.size(); ++s) tab[s] = e->inst[s].dev;
  if ((rc = e->TAB.ensure(sizeof(EnsInst) * std::max<size_t>(tab.size(), 1), e->st))) return rc;
  if (!tab.empty())
    GC_CUDA(cudaMemcpyAsync(e->TAB.p, tab.data(), sizeof(EnsInst) * tab.size(), cudaMemcpyHostToDevice, e->st));
  // tile tables of the tiled list build (one per cells-per-block choice) and
  // the particles-per-cell estimate that sizes its buffers
  {
    const size_t ni = e->inst.size();
    std::vector<int32_t> tiles(4 * (ni + 1));
    for (int c = 0; c < 4; ++c) {
      int64_t acc = 0;
      for (size_t si = 0; si < ni; ++si) {
        const EnsInst& I = e->inst[si].dev;
        tiles[c * (ni + 1) + si] = (int32_t)acc;
        acc += (int64_t)((I.nc[0] + kCpbs[c] - 1) / kCpbs[c]) * I.nc[1] * I.nc[2];
      }
      tiles[c * (ni + 1) + ni] = (int32_t)acc;
      e->ntiles[c] = (int)acc;
    }
    double ppc = 1.0;
    for (const EnsHostInst& h : e->inst)
      if (h.prm.dx > 0) ppc = std::max(ppc, std::pow(h.prm.H / h.prm.dx, (double)e->D));
    e->ppc = ppc;
    if ((rc = e->TILES.ensure(sizeof(int32_t) * tiles.size(), e->st))) return rc;
    GC_CUDA(cudaMemcpyAsync(e->TILES.p, tiles.data(), sizeof(int32_t) * tiles.size(), cudaMemcpyHostToDevice,
                            e->st));
    GC_CUDA(cudaStreamSynchronize(e->st));
  }
  {
    // per-instance list flags in the new packing order
    const size_t ni = std::max<size_t>(e->inst.size(), 1);
    std::vector<int32_t> rb(ni, 1), nreb(ni, 0);
    for (size_t si = 0; si < e->inst.size(); ++si) {
      rb[si] = e->inst[si].rb;
      nreb[si] = e->inst[si].nreb;
    }
    if ((rc = e->RB.ensure(sizeof(int32_t) * ni, e->st))) return rc;
    if ((rc = e->NREB.ensure(sizeof(int32_t) * ni, e->st))) return rc;
    if ((rc = e->DMAX.ensure(sizeof(unsigned) * ni, e->st, true))) return rc;
    if ((rc = e->SDMAX.ensure(sizeof(unsigned) * ni, e->st, true))) return rc;
    GC_CUDA(cudaMemcpyAsync(e->RB.p, rb.data(), sizeof(int32_t) * ni, cudaMemcpyHostToDevice, e->st));
    GC_CUDA(cudaMemcpyAsync(e->NREB.p, nreb.data(), sizeof(int32_t) * ni, cudaMemcpyHostToDevice, e->st));
    GC_CUDA(cudaMemsetAsync(e->DMAX.p, 0, sizeof(unsigned) * ni, e->st));
    GC_CUDA(cudaMemsetAsync(e->SDMAX.p, 0, sizeof(unsigned) * ni, e->st));
    GC_CUDA(cudaStreamSynchronize(e->st));
  }
  std::vector<int32_t> isteps(e->inst.size());
  for (size_t s = 0; s < e->inst.size(); ++s) isteps[s] = (int32_t)(e->inst[s].steps % 2000000000LL);
  if ((rc = e->ISTEP.ensure(sizeof(int32_t) * std::max<size_t>(isteps.size(), 1), e->st))) return rc;
  if (!isteps.empty())
    GC_CUDA(cudaMemcpyAsync(e->ISTEP.p, isteps.data(), sizeof(int32_t) * isteps.size(), cudaMemcpyHostToDevice,
                            e->st));
  for (size_t s = 0; s < e->inst.size(); ++s) {
    EnsHostInst& h = e->inst[s];
    if (h.n == 0 || (h.filled_off == h.p_off && h.filled_idx == (int64_t)s)) continue;
    k_fill_i32<<<nblocks(h.n, 256), 256, 0, e->st>>>(e->INST.as<int32_t>() + h.p_off, h.n, (int32_t)s);
    GC_LAUNCHED();
    h.filled_off = h.p_off;
    h.filled_idx = (int64_t)s;
  }
  GC_CUDA(cudaStreamSynchronize(e->st));
  e->gen += 1;
  graphs_free(e);
  return GCSPH_OK;
}

// the tiled list build's kernel for (lanes, staging depth)
using TileKern = void (*)(EnsArr, const EnsInst*, const int*, int, int, int);
template <int D>
TileKern tile_kernel(int L, int depth) {
  switch (L) {
    case 2: return depth == 2 ? k_ens_nlist_tile<D, 2, 2> : k_ens_nlist_tile<D, 2, 1>;
    case 4: return depth == 2 ? k_ens_nlist_tile<D, 4, 2> : k_ens_nlist_tile<D, 4, 1>;
    case 8: return depth == 2 ? k_ens_nlist_tile<D, 8, 2> : k_ens_nlist_tile<D, 8, 1>;
    default: return depth == 2 ? k_ens_nlist_tile<D, 1, 2> : k_ens_nlist_tile<D, 1, 1>;
  }
}

int ens_occupancy(gcsph_ens* e) {
  if (e->sms) return GCSPH_OK;
  int dev = 0;
  GC_CUDA(cudaGetDevice(&dev));
  GC_CUDA(cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, dev));
  for (int t = 0; t < 3; ++t) {
    int b = 0;
    if (e->D == 2)
      GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ens_stage<2, 2>, kTpbs[t], 0));
    else
      GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_ens_stage<3, 2>, kTpbs[t], 0));
    e->occ[t] = std::max(b, 1);
    int b2 = 0;
    if (e->D == 2)
      GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_ens_nlist<2, 4>, kTpbs[t], 0));
    else
      GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_ens_nlist<3, 4>, kTpbs[t], 0));
    e->occ_nl[t] = std::max(b2, 1);
    int b3 = 0;
    if (e->D == 2)
      GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b3, k_ens_xsph<2>, kTpbs[t], 0));
    else
      GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b3, k_ens_xsph<3>, kTpbs[t], 0));
    e->occ_x[t] = std::max(b3, 1);
  }
  const int lanes[4] = {1, 2, 4, 8};
  for (int l = 0; l < 4; ++l)
    for (int dp = 1; dp <= 2; ++dp) {
      if (e->D == 2)
        GC_CUDA(cudaFuncSetAttribute(tile_kernel<2>(lanes[l], dp), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     96 * 1024));
      else
        GC_CUDA(cudaFuncSetAttribute(tile_kernel<3>(lanes[l], dp), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     96 * 1024));
    }
  return GCSPH_OK;
}

int tpb_index(int tpb) {
  for (int t = 0; t < 3; ++t)
    if (kTpbs[t] == tpb) return t;
  return 1;
}

// one step of every instance: bin, re-sort, predictor pass, corrector pass
// grid of a grid-stride pass over `want` blocks' worth of rows, with `slots`
// blocks resident on the GPU: every block once from four waves up (the block
// scheduler balances rows of unequal length); below that a persistent grid of
// the resident blocks, where a partial second wave would leave SMs idle
// (measured on GB300 for xsphcorr!: 0.95 -> 0.83 ms at 2 M 3-D particles, 8.7
// waves; persistent 0.15 ms against 0.18 at 0.4 M, 1.7 waves)
int wave_grid(int64_t want, int64_t slots) {
  return (int)std::max<int64_t>(1, want >= 4 * slots ? want : std::min<int64_t>(want, slots));
}

template <int D>
int ens_enqueue_step(gcsph_ens* e, cudaStream_t st, int tpb) {
  const int64_t N = e->N;
  const EnsInst* T = e->TAB.as<EnsInst>();
  GC_CUDA(cudaMemsetAsync(e->COUNT.p, 0, sizeof(int32_t) * e->K, st));
  const double* x2 = D == 3 ? e->X[e->cur][2].as<double>() : e->X[e->cur][0].as<double>();
  k_ens_key<D><<<nblocks(N, 256), 256, 0, st>>>(N, e->INST.as<int32_t>(), e->X[e->cur][0].as<double>(),
                                                 e->X[e->cur][1].as<double>(), x2, T, e->RB.as<int>(),
                                                 e->SKEY.as<int32_t>(), e->KEY.as<int32_t>(),
                                                 e->SLOT.as<int32_t>(), e->COUNT.as<int32_t>());
  GC_LAUNCHED();
  int rc = exclusive_scan_i32_to_i32(e->COUNT.as<int32_t>(), e->CELLSTART.as<int32_t>(), e->K,
                                     e->SCRATCH.as<int64_t>(), st);
  if (rc) return rc;
  k_ens_scatter<<<nblocks(N, 256), 256, 0, st>>>(N, e->KEY.as<int32_t>(), e->SLOT.as<int32_t>(),
                                                 e->CELLSTART.as<int32_t>(), e->TMP.as<int32_t>());
  GC_LAUNCHED();
  k_ens_rank<<<nblocks(N, 256), 256, 0, st>>>(N, e->TMP.as<int32_t>(), e->KEY.as<int32_t>(),
                                              e->CELLSTART.as<int32_t>(), e->ID[e->cur].as<int32_t>(),
                                              e->PERM.as<int32_t>());
  GC_LAUNCHED();
  float* o2 = D == 3 ? e->OFF[2].as<float>() : e->OFF[0].as<float>();
  k_ens_permute<D><<<nblocks(N, 256), 256, 0, st>>>(N, e->PERM.as<int32_t>(), e->KEY.as<int32_t>(),
                                                     e->INST.as<int32_t>(), T, ens_state(e, e->cur),
                                                     ens_state(e, e->cur ^ 1), e->SKEY.as<int32_t>(),
                                                     e->OFF[0].as<float>(), e->OFF[1].as<float>(), o2,
                                                     e->R1.as<float4>(), e->RB.as<int>(), e->OB[0].as<float>(),
                                                     e->OB[1].as<float>(),
                                                     D == 3 ? e->OB[2].as<float>() : e->OB[0].as<float>());
  GC_LAUNCHED();
  e->cur ^= 1;
  const int t = tpb_index(tpb);
  const int64_t want = (N + tpb - 1) / tpb;
  const int grid = wave_grid(want, (int64_t)e->sms * e->occ[t]);
  EnsArr A = ens_arr(e);
  timer_begin(T_PAIRS, st);
  if (e->nl_cpb > 0) {
    // tiles of nl_cpb cells per block, neighbourhood staged in shared memory
    const int ci = cpb_index(e->nl_cpb);
    const int cap = tile_cap(e, e->nl_cpb, e->nl_depth);
    const size_t smem = sizeof(float) * (size_t)D * cap * e->nl_depth;
    const TileKern k = tile_kernel<D>(e->nl_lanes, e->nl_depth);
    int b = 0;
    GC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, TILE_TPB, smem));
    const int ni = (int)e->inst.size();
    const int g3 = std::max(1, std::min(e->ntiles[ci], e->sms * std::max(b, 1)));
    k<<<g3, TILE_TPB, smem, st>>>(A, T, e->TILES.as<int32_t>() + (size_t)ci * (ni + 1), ni, e->nl_cpb, cap);
  } else {
    // L lanes per particle in the list build (the list is the same for every L)
    const int L = e->nl_lanes;
    const int64_t gwant = (N * L + tpb - 1) / tpb;
    const int g2 = wave_grid(gwant, (int64_t)e->sms * e->occ_nl[t]);
    switch (L) {
      case 2: k_ens_nlist<D, 2><<<g2, tpb, 0, st>>>(A, T); break;
      case 4: k_ens_nlist<D, 4><<<g2, tpb, 0, st>>>(A, T); break;
      case 8: k_ens_nlist<D, 8><<<g2, tpb, 0, st>>>(A, T); break;
      default: k_ens_nlist<D, 1><<<g2, tpb, 0, st>>>(A, T); break;
    }
  }
  GC_LAUNCHED();
  timer_end(T_PAIRS, st);
  const int64_t swant = (N * stage_lanes<D>() + tpb - 1) / tpb;
  // one block per tpb / L particles, not a persistent grid: the block
  // scheduler balances rows of unequal length, and the particles in flight
  // stay one contiguous window of the cell order (measured on GB300: the
  // 3-D dam break's stage passes 8% faster at 0.4 M and 2 M particles)
  const int sgrid = (int)std::max<int64_t>(1, swant);
  timer_begin(T_STAGE1, st);
  if (A.rmin2)
    k_ens_stage<D, 1, true><<<sgrid, tpb, 0, st>>>(A, T);
  else
    k_ens_stage<D, 1, false><<<sgrid, tpb, 0, st>>>(A, T);
  GC_LAUNCHED();
  timer_end(T_STAGE1, st);
  timer_begin(T_STAGE2, st);
  k_ens_stage<D, 2><<<sgrid, tpb, 0, st>>>(A, T);
  GC_LAUNCHED();
  timer_end(T_STAGE2, st);
  const int32_t ninst = (int32_t)e->inst.size();
  if (e->any_dpc) {
    timer_begin(T_DPC, st);
    if (A.rmin2) {
      k_ens_disp<D, true><<<nblocks(N, 256), 256, 0, st>>>(A, T, e->SDMAX.as<unsigned>());
      GC_LAUNCHED();
    }
    k_ens_dpc<D><<<grid, tpb, 0, st>>>(A, T);
    GC_LAUNCHED();
    k_ens_dpc_apply<D><<<nblocks(N, 256), 256, 0, st>>>(A, T);
    GC_LAUNCHED();
    timer_end(T_DPC, st);
  }
  if (e->any_xsph) {
    timer_begin(T_XSPH, st);
    k_ens_xsph<D><<<wave_grid(want, (int64_t)e->sms * e->occ_x[t]), tpb, 0, st>>>(A, T);
    GC_LAUNCHED();
    timer_end(T_XSPH, st);
  }
  if (e->any_cspm) {
    timer_begin(T_CSPM, st);
    k_ens_cspm<D><<<grid, tpb, 0, st>>>(A, T, e->ISTEP.as<int32_t>());
    GC_LAUNCHED();
    k_ens_cspm_apply<<<nblocks(N, 256), 256, 0, st>>>(N, e->INST.as<int32_t>(), T, e->ISTEP.as<int32_t>(),
                                                      e->DRH.as<float>(), e->DR[e->cur].as<float>(), A.ovf);
    GC_LAUNCHED();
    timer_end(T_CSPM, st);
  }
  k_ens_disp<D, false><<<nblocks(N, 256), 256, 0, st>>>(A, T, e->DMAX.as<unsigned>());
  GC_LAUNCHED();
  k_ens_tick<<<nblocks(std::max(ninst, 1), 128), 128, 0, st>>>(ninst, e->ISTEP.as<int32_t>(), A.ovf,
                                                                  A.ovf + 2, T, e->RB.as<int>(),
                                                                  e->NREB.as<int>(), e->DMAX.as<unsigned>(),
                                                                  e->SDMAX.as<unsigned>());
  GC_LAUNCHED();
  return GCSPH_OK;
}

int enqueue_step(gcsph_ens* e, cudaStream_t st, int tpb) {
  return e->D == 2 ? ens_enqueue_step<2>(e, st, tpb) : ens_enqueue_step<3>(e, st, tpb);
}

// Launch shapes, tuned in three phases on real steps (the arithmetic per
// particle does not depend on the launch shape, so tuning steps are ordinary
// steps); each candidate runs two steps and the second is timed:
//   1. block size of the pair passes (6 steps);
//   2. lanes per particle of the list build (8 steps);
//   3. the list build's tiling: a thread group per particle against tiles of
//      cells-per-block cells staged in shared memory, three tile sizes at
//      staging depth 1, then the best at depth 2 (10 steps).
// A phase runs when the call has the steps for it; the rest wait for a later
// call.  A particle count that moves past 2x of the tuned one starts over.
int ens_autotune(gcsph_ens* e, int32_t budget, int32_t* steps_used) {
  *steps_used = 0;
  if (e->tpb_fixed) return GCSPH_OK;
  if (e->tune_phase > 0 && !(e->N <= 2 * e->tuned_n && 2 * e->N >= e->tuned_n)) e->tune_phase = 0;
  if (e->tune_phase >= 3) return GCSPH_OK;
  if (!e->tpb) e->tpb = 256;
  cudaEvent_t a, b;
  GC_CUDA(cudaEventCreate(&a));
  GC_CUDA(cudaEventCreate(&b));
  int rc = GCSPH_OK;
  auto timed = [&](int tpb) -> float {
    float last = 0.f;
    for (int r = 0; r < 2 && rc == GCSPH_OK; ++r) {
      cudaEventRecord(a, e->st);
      rc = enqueue_step(e, e->st, tpb);
      cudaEventRecord(b, e->st);
      cudaEventSynchronize(b);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      last = ms;  // the first run of each shape warms caches
      *steps_used += 1;
    }
    return last;
  };
  if (e->tune_phase == 0 && budget - *steps_used >= 6) {
    float best = 1e30f;
    int pick = 256;
    for (int t = 0; t < 3 && rc == GCSPH_OK; ++t) {
      const float ms = timed(kTpbs[t]);
      if (ms < best) {
        best = ms;
        pick = kTpbs[t];
      }
    }
    e->tpb = pick;
    e->tuned_n = e->N;
    e->tune_phase = 1;
  }
  if (e->tune_phase == 1 && e->nl_fixed) e->tune_phase = 3;
  if (rc == GCSPH_OK && e->tune_phase == 1 && budget - *steps_used >= 8) {
    const int lanes[4] = {1, 2, 4, 8};
    const int cpb0 = e->nl_cpb;
    e->nl_cpb = 0;
    float best = 1e30f;
    int pick = e->nl_lanes;
    for (int t = 0; t < 4 && rc == GCSPH_OK; ++t) {
      e->nl_lanes = lanes[t];
      const float ms = timed(e->tpb);
      if (ms < best) {
        best = ms;
        pick = lanes[t];
      }
    }
    e->nl_lanes = pick;
    e->nl_cpb = cpb0;
    e->tune_phase = 2;
  }
  if (rc == GCSPH_OK && e->tune_phase == 2 && budget - *steps_used >= 10) {
    const int c2[3] = {4, 8, 16}, c3[3] = {2, 4, 8};
    const int* cpbs = e->D == 2 ? c2 : c3;
    e->nl_cpb = 0;
    e->nl_depth = 1;
    float best = timed(e->tpb);
    int pick = 0, pickd = 1;
    for (int t = 0; t < 3 && rc == GCSPH_OK; ++t) {
      e->nl_cpb = cpbs[t];
      const float ms = timed(e->tpb);
      if (ms < best) {
        best = ms;
        pick = cpbs[t];
      }
    }
    if (pick > 0 && rc == GCSPH_OK) {
      e->nl_cpb = pick;
      e->nl_depth = 2;
      if (timed(e->tpb) < best) pickd = 2;
    }
    e->nl_cpb = pick;
    e->nl_depth = pickd;
    e->tune_phase = 3;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rc;
}

int ens_run_graph(gcsph_ens* e, int32_t n) {
  EnsGraph* g = nullptr;
  const int timing = timing_on() ? 1 : 0;
  for (EnsGraph& c : e->graphs)
    if (c.exec && c.n_steps == n && c.N == e->N && c.K == e->K && c.gen == e->gen && c.cur == e->cur &&
        c.tpb == e->tpb && c.timing == timing && c.nl_lanes == e->nl_lanes && c.nl_cpb == e->nl_cpb &&
        c.nl_depth == e->nl_depth && c.nl_cap == e->nl_cap_fix && c.dpc_bound == (int)e->dpc_bound)
      g = &c;
  if (!g) {
    g = &e->graphs[0];
    for (EnsGraph& c : e->graphs)
      if (!c.exec || c.used < g->used) g = &c;
    graph_free(*g);
    if (!e->cap) GC_CUDA(cudaStreamCreateWithFlags(&e->cap, cudaStreamNonBlocking));
    const int cur0 = e->cur;
    const unsigned long long l0 = gcsph_launch_count();
    GC_CUDA(cudaStreamBeginCapture(e->cap, cudaStreamCaptureModeThreadLocal));
    timer_capture_to(&g->timers);
    int rc = GCSPH_OK;
    for (int32_t it = 0; it < n && rc == GCSPH_OK; ++it) rc = enqueue_step(e, e->cap, e->tpb);
    timer_capture_to(nullptr);
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(e->cap, &graph);
    const unsigned long long l1 = gcsph_launch_count();
    count_launch(-(int)(l1 - l0));
    const int cur1 = e->cur;
    e->cur = cur0;
    if (rc == GCSPH_OK && ce != cudaSuccess) rc = cuda_fail(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
    if (rc == GCSPH_OK) {
      ce = cudaGraphInstantiate(&g->exec, graph, 0);
      if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaGraphInstantiate", __FILE__, __LINE__);
    }
    if (graph) cudaGraphDestroy(graph);
    if (rc != GCSPH_OK) {
      cudaGetLastError();
      graph_free(*g);
      return rc;
    }
    g->timing = timing;
    g->nl_lanes = e->nl_lanes;
    g->nl_cpb = e->nl_cpb;
    g->nl_depth = e->nl_depth;
    g->nl_cap = e->nl_cap_fix;
    g->dpc_bound = (int)e->dpc_bound;
    g->n_steps = n;
    g->N = e->N;
    g->K = e->K;
    g->gen = e->gen;
    g->cur = cur0;
    g->tpb = e->tpb;
    g->launches = (long long)(l1 - l0);
    (void)cur1;
    e->n_captures += 1;
  }
  g->used = ++e->clock;
  GC_CUDA(cudaGraphLaunch(g->exec, e->st));
  GC_CUDA(cudaStreamSynchronize(e->st));
  count_launch((int)g->launches);
  timer_account(g->timers);
  if (n & 1) e->cur ^= 1;
  e->n_replays += 1;
  return GCSPH_OK;
}


int ens_run(gcsph_ens* e, int32_t n) {
  if (n <= 0 || e->N == 0) return GCSPH_OK;
  if (!e->use_graphs) {
    for (int32_t it = 0; it < n; ++it) {
      int rc = enqueue_step(e, e->st, e->tpb);
      if (rc) return rc;
    }
    GC_CUDA(cudaStreamSynchronize(e->st));
    timer_collect();
    return GCSPH_OK;
  }
  return ens_run_graph(e, n);
}

EnsHostInst* find_slot(gcsph_ens* e, int32_t slot, size_t* pos = nullptr) {
  for (size_t s = 0; s < e->inst.size(); ++s)
    if (e->inst[s].slot == slot) {
      if (pos) *pos = s;
      return &e->inst[s];
    }
  return nullptr;
}

}  // namespace

extern "C" {

int ens_create(int32_t D, void* stream, gcsph_ens** out) {
  if (!out) return fail(GCSPH_EINVAL, "null argument");
  *out = nullptr;
  if (D != 2 && D != 3) return fail(GCSPH_EINVAL, "wrong dimention: D=%d (2 or 3)", (int)D);
  gcsph_ens* e = new gcsph_ens();
  e->D = D;
  e->skin = D == 2 ? 0.05 : 0.025;  // the fastest measured on GB300 (256-instance 2-D, 3-D dam break)
  e->st = (cudaStream_t)stream;
  int rc = ens_occupancy(e);
  if (rc) {
    delete e;
    return rc;
  }
  *out = e;
  return GCSPH_OK;
}

void ens_destroy(gcsph_ens* e) {
  if (!e) return;
  cudaStreamSynchronize(e->st);
  graphs_free(e);
  if (e->cap) cudaStreamDestroy(e->cap);
  for (int b = 0; b < 2; ++b) {
    for (int d = 0; d < 3; ++d) {
      e->X[b][d].release();
      e->V[b][d].release();
      e->DXB[b][d].release();
      e->DVB[b][d].release();
    }
    e->DR[b].release();
    e->DRB[b].release();
    e->PT[b].release();
    e->ID[b].release();
  }
  DevBuf* one[] = {&e->INST, &e->KEY, &e->SLOT, &e->TMP, &e->PERM, &e->SKEY, &e->DRH, &e->COUNT, &e->CELLSTART,
                   &e->SCRATCH, &e->TAB, &e->MOVES, &e->OUT, &e->ISTEP, &e->NL, &e->NLC, &e->FLAGS,
                   &e->R1, &e->R2};
  for (DevBuf* b : one) b->release();
  for (int d = 0; d < 3; ++d) {
    e->OFF[d].release();
    e->OFFH[d].release();
    e->VH[d].release();
    e->OFFN[d].release();
  }
  delete e;
}

int ens_bytes_per_particle(int32_t D, int64_t* bytes) {
  if (!bytes || (D != 2 && D != 3)) return fail(GCSPH_EINVAL, "bad argument");
  // 2 x (x f64, v f32, x and v base differences f32) per dim + 2 x (δρ,
  // δρ base, ptype, id) + inst, key, slot, tmp, perm, skey + (off, offh, vh,
  // offn) per dim + δρ½, plus about one cell per particle
  // + the step's neighbour list (64 entries in 2-D, 256 in 3-D, 4 B each) and its length
  *bytes = 2 * D * (8 + 4 + 8) + 2 * 16 + 6 * 4 + D * 16 + 4 + 8 + (D == 2 ? 64 : 256) * 4 + 4 +
           16 * (D == 2 ? 4 : 5) +  // packed records of the stages
           64 +                     // and of the correction passes
           D * 4 +                  // offsets at the last list build
           4;                       // the row's smallest r² (dpcreg!'s row bound)
  return GCSPH_OK;
}

int ens_add(gcsph_ens* e, int64_t n, const double* x, const double* v, const double* rho, const int32_t* ptype,
            const gcsph_ens_params* p, int32_t* slot_out) {
  if (!e || !x || !rho || !ptype || !p || !slot_out) return fail(GCSPH_EINVAL, "null argument");
  if (n <= 0 || n > (int64_t)INT32_MAX / 2) return fail(GCSPH_EINVAL, "particle count %lld", (long long)n);
  if (!(p->H > 0) || !(p->dt > 0) || p->gamma <= 0) return fail(GCSPH_EINVAL, "H, dt and gamma must be positive");
  const int D = e->D;
  EnsHostInst h{};
  h.slot = e->next_slot++;
  h.n = n;
  h.prm = *p;
  h.steps = 0;
  EnsInst& I = h.dev;
  memset(&I, 0, sizeof(I));
  // cells (and the list radius) of H (1 + skin): the list holds every pair
  // within H until some particle has moved skin H / 2
  const double cs = p->H * (1.0 + e->skin);
  I.reuse = e->skin > 0.0;
  I.LR2 = (float)(cs * cs);
  I.dthr2 = (float)((0.49 * e->skin * p->H) * (0.49 * e->skin * p->H));
  int64_t ncell = 1;
  for (int d = 0; d < 3; ++d) {
    if (d < D) {
      if (!(p->grid_max[d] > p->grid_min[d])) return fail(GCSPH_EINVAL, "empty grid in dimension %d", d + 1);
      I.origin[d] = p->grid_min[d];
      const double span = p->grid_max[d] - p->grid_min[d];
      const double nc = floor(span / cs) + 1.0;
      if (nc > 1e8) return fail(GCSPH_EINVAL, "grid too fine");
      I.nc[d] = (int)nc;
    } else {
      I.origin[d] = 0.0;
      I.nc[d] = 1;
    }
    ncell *= I.nc[d];
  }
  if (ncell > (int64_t)INT32_MAX / 2) return fail(GCSPH_EINVAL, "grid of %lld cells", (long long)ncell);
  h.ncell = ncell;
  I.cs = cs;
  I.csinv = 1.0 / cs;
  I.csf = (float)cs;
  I.dt = p->dt;
  I.gamma = p->gamma;
  I.cspmn = p->cspmn > 0 ? p->cspmn : 0;
  I.use_visc = p->nu > 0;
  I.use_pF = p->s > 0;
  I.H2 = (float)(p->H * p->H);
  I.h = (float)p->h;
  I.Hinv = (float)(1.0 / p->H);
  I.nW = (float)(D == 2 ? wc2_norm_w<2>(1.0 / p->H) : wc2_norm_w<3>(1.0 / p->H));
  I.nDW = (float)(D == 2 ? wc2_norm_dw<2>(1.0 / p->H) : wc2_norm_dw<3>(1.0 / p->H));
  I.m0 = (float)p->m0;
  I.rho0 = (float)p->rho0;
  I.c0 = (float)p->c0;
  I.P0 = (float)(p->c0 * p->c0 * p->rho0 / (double)p->gamma);
  I.alpha = (float)p->alpha;
  I.DDTkh = (float)(2.0 * p->h * p->delta * p->c0);
  I.DDTgz = (float)(p->rho0 * p->g / ((p->c0 * p->c0 * p->rho0) / (double)p->gamma));
  I.eta2 = (float)((0.1 * p->h) * (0.1 * p->h));
  I.g = (float)p->g;
  I.nu = (float)p->nu;
  I.s = (float)p->s;
  I.twoh = (float)(2.0 * p->h);
  I.pfc = (float)(1.5 * GCSPH_PI64);
  I.hp1 = (float)(0.1 * p->h);
  const double r01 = 2.0 * p->dx;
  I.fb_d[0] = 0.4f;
  I.fb_r0[0] = (float)r01;
  I.fb_eta2[0] = (float)(0.01 * r01 * r01);
  I.fb_d[1] = (float)p->bound_D;
  I.fb_r0[1] = (float)p->bound_l;
  I.fb_eta2[1] = (float)(0.01 * p->bound_l * p->bound_l);
  I.use_dpc = p->dpc_l0 > 0;
  if (I.use_dpc) {
    const double l0inv = 1.0 / p->dpc_l0;
    const double nW = D == 2 ? wc2_norm_w<2>(l0inv) : wc2_norm_w<3>(l0inv);
    I.dpc_l0inv = (float)l0inv;
    I.dpc_nW = (float)nW;
    I.dpc_whinv = (float)(1.0 / wc2_w(0.5, nW));
    I.dpc_kernlim = (float)gcsph_dpckernlim(D);
    I.dpc_eta2 = (float)((0.1 * p->dpc_l0) * (0.1 * p->dpc_l0));
    I.dpc_pmin = (float)p->dpc_pmin;
    I.dpc_pmax = (float)p->dpc_pmax;
    I.dpc_lambda = (float)p->dpc_lambda;
    // the bound's margin: 1e-3 l0, and 1e-5 cell edges for the FP32 offsets
    // (their rounding is a few 1e-7 cell edges)
    I.dpc_skip = (float)(p->dpc_l0 * (1.0 + 1e-3) + 1e-5 * I.cs);
  }
  I.use_xsph = p->xsph_eps > 0;
  I.xsph_c = (float)(2.0 * p->m0 * p->xsph_eps);
  const double a = 1.0 / (double)p->gamma;
  const double c1 = a, c2 = c1 * (a - 1.0) / 2.0, c3 = c2 * (a - 2.0) / 3.0, c4 = c3 * (a - 3.0) / 4.0;
  I.pc[0] = (float)c1;
  I.pc[1] = (float)c2;
  I.pc[2] = (float)c3;
  I.pc[3] = (float)c4;
  I.rho0inv = (float)(1.0 / p->rho0);
  I.m0inv = (float)(1.0 / p->m0);
  I.dwc = (float)(-20.0 * (D == 2 ? wc2_norm_dw<2>(1.0 / p->H) : wc2_norm_dw<3>(1.0 / p->H)) / p->H);
  I.pfcr = (float)(1.5 * GCSPH_PI64 / (2.0 * p->h));
  I.kddt = (float)(2.0 * p->h * p->delta * p->c0 * p->m0);
  I.kav = (float)(2.0 * p->alpha * p->c0 * p->h * p->m0);
  I.kvisc = (float)(4.0 * p->nu * p->m0);
  I.kpf = (float)(p->s / p->m0);
  I.kA = make_float4(I.H2, I.Hinv, I.dwc, I.csf);
  I.kB = make_float4(I.rho0, I.eta2, I.m0, I.DDTgz);
  I.kC = make_float4(I.kddt, I.kav, I.kvisc, 0.f);
  I.kD = make_float4(I.pfcr, I.hp1, I.twoh, I.kpf);
  I.kE = make_float4(I.pc[0], I.pc[1], I.pc[2], I.pc[3]);
  for (int st = 0; st < 2; ++st) I.kFB[st] = make_float4(I.fb_d[st], I.fb_r0[st], I.fb_eta2[st], 0.f);
  // host staging in the engine's types
  std::vector<float> vf((size_t)D * n, 0.f), drf((size_t)n);
  std::vector<int32_t> ids((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    drf[i] = (float)(rho[i] - p->rho0);
    ids[i] = (int32_t)i;
  }
  if (v)
    for (int64_t i = 0; i < (int64_t)D * n; ++i) vf[i] = (float)v[i];
  const int64_t at = e->N;
  int rc;
  if ((rc = ens_reserve(e, at + n))) return rc;
  const int b = e->cur;
  for (int d = 0; d < D; ++d) {
    GC_CUDA(cudaMemcpyAsync(e->X[b][d].as<double>() + at, x + (size_t)d * n, sizeof(double) * n,
                            cudaMemcpyHostToDevice, e->st));
    GC_CUDA(cudaMemcpyAsync(e->V[b][d].as<float>() + at, vf.data() + (size_t)d * n, sizeof(float) * n,
                            cudaMemcpyHostToDevice, e->st));
  }
  GC_CUDA(cudaMemcpyAsync(e->DR[b].as<float>() + at, drf.data(), sizeof(float) * n, cudaMemcpyHostToDevice, e->st));
  GC_CUDA(cudaMemcpyAsync(e->DRB[b].as<float>() + at, drf.data(), sizeof(float) * n, cudaMemcpyHostToDevice, e->st));
  for (int d = 0; d < D; ++d) {
    GC_CUDA(cudaMemsetAsync(e->DXB[b][d].as<float>() + at, 0, sizeof(float) * n, e->st));
    GC_CUDA(cudaMemsetAsync(e->DVB[b][d].as<float>() + at, 0, sizeof(float) * n, e->st));
  }
  GC_CUDA(cudaMemcpyAsync(e->PT[b].as<int32_t>() + at, ptype, sizeof(int32_t) * n, cudaMemcpyHostToDevice, e->st));
  GC_CUDA(cudaMemcpyAsync(e->ID[b].as<int32_t>() + at, ids.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice,
                          e->st));
  GC_CUDA(cudaStreamSynchronize(e->st));
  if ((rc = ens_pull_flags(e))) return rc;
  e->inst.push_back(h);
  if ((rc = ens_relayout(e))) {
    e->inst.pop_back();
    ens_relayout(e);
    return rc;
  }
  *slot_out = h.slot;
  return GCSPH_OK;
}

int ens_remove(gcsph_ens* e, int32_t slot) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  size_t pos = 0;
  if (!find_slot(e, slot, &pos)) return fail(GCSPH_EINVAL, "no instance in slot %d", (int)slot);
  int rc;
  if ((rc = ens_pull_flags(e))) return rc;
  std::vector<Move> mv;
  std::vector<int64_t> old_key;  // key offsets before the removal, of the instances that stay
  int64_t p = 0;
  for (size_t s = 0; s < e->inst.size(); ++s) {
    if (s == pos) continue;
    mv.push_back({p, e->inst[s].p_off, e->inst[s].n});
    old_key.push_back(e->inst[s].key_off);
    p += e->inst[s].n;
  }
  e->inst.erase(e->inst.begin() + (long)pos);
  if (p > 0) {
    if ((rc = e->MOVES.ensure(sizeof(Move) * mv.size(), e->st))) return rc;
    GC_CUDA(cudaMemcpyAsync(e->MOVES.p, mv.data(), sizeof(Move) * mv.size(), cudaMemcpyHostToDevice, e->st));
    const Move* M = e->MOVES.as<Move>();
    const int nb = nblocks(p, 256);
    k_ens_repack<<<nb, 256, 0, e->st>>>((int)mv.size(), M, p, e->D, ens_state(e, e->cur),
                                        ens_state(e, e->cur ^ 1));
    GC_LAUNCHED();
    e->cur ^= 1;
    // what the instances keep between list builds moves with them, through
    // the sort's scratch: cell keys, build offsets, list rows
    int32_t* tmp = e->TMP.as<int32_t>();
    auto move32 = [&](void* buf) -> int {
      k_ens_repack32<<<nb, 256, 0, e->st>>>((int)mv.size(), M, p, (const int32_t*)buf, tmp);
      GC_LAUNCHED();
      GC_CUDA(cudaMemcpyAsync(buf, tmp, sizeof(int32_t) * p, cudaMemcpyDeviceToDevice, e->st));
      return GCSPH_OK;
    };
    if ((rc = move32(e->SKEY.p))) return rc;
    for (int d = 0; d < e->D; ++d)
      if ((rc = move32(e->OB[d].p))) return rc;
    if (e->NL.p && e->NLC.p) {
      if ((rc = move32(e->NLC.p))) return rc;
      for (int q = 0; q < e->nls; ++q)
        if ((rc = move32(e->NL.as<int32_t>() + (size_t)q * (size_t)e->nl_cap))) return rc;
    }
  }
  if ((rc = ens_relayout(e))) return rc;
  if (p > 0) {
    std::vector<int32_t> delta(e->inst.size());
    for (size_t s = 0; s < e->inst.size(); ++s) delta[s] = (int32_t)(e->inst[s].key_off - old_key[s]);
    if ((rc = e->SCRATCH.ensure(sizeof(int64_t) * std::max<size_t>(delta.size(), 1), e->st))) return rc;
    GC_CUDA(cudaMemcpyAsync(e->SCRATCH.p, delta.data(), sizeof(int32_t) * delta.size(), cudaMemcpyHostToDevice,
                            e->st));
    k_ens_shift_keys<<<nblocks(p, 256), 256, 0, e->st>>>(p, e->INST.as<int32_t>(), e->SCRATCH.as<int32_t>(),
                                                         e->SKEY.as<int32_t>());
    GC_LAUNCHED();
    GC_CUDA(cudaStreamSynchronize(e->st));
  }
  return GCSPH_OK;
}

int ens_set_stream(gcsph_ens* e, void* stream) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if ((cudaStream_t)stream == e->st) return GCSPH_OK;
  GC_CUDA(cudaStreamSynchronize(e->st));  // the old stream's work is done before the next call's starts
  e->st = (cudaStream_t)stream;
  return GCSPH_OK;
}

int ens_step(gcsph_ens* e, int32_t n) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if (n < 0) return fail(GCSPH_EINVAL, "n must be >= 0");
  if (e->N == 0 || n == 0) return GCSPH_OK;
  int rc;
  if ((rc = ens_reserve_list(e, e->nls ? e->nls : (e->D == 2 ? 64 : 256)))) return rc;
  if (e->lists_lost) {
    // no list survived: every instance builds one at its next step
    GC_CUDA(cudaMemsetAsync(e->RB.p, 0x01, sizeof(int32_t) * e->inst.size(), e->st));
    e->lists_lost = false;
  }
  int32_t left = n;
  int guard = 0;
  while (left > 0) {
    // a call: tuning steps (eager) and the rest (a graph), with the list
    // overflow flag cleared; the flags say how many steps completed
    GC_CUDA(cudaMemsetAsync(e->FLAGS.p, 0, sizeof(int) * 4, e->st));
    int32_t used = 0;
    if ((rc = ens_autotune(e, left, &used))) return rc;
    if (left - used > 0 && (rc = ens_run(e, left - used))) return rc;
    int fl[4];
    GC_CUDA(cudaMemcpyAsync(fl, e->FLAGS.p, sizeof(fl), cudaMemcpyDeviceToHost, e->st));
    GC_CUDA(cudaStreamSynchronize(e->st));
    const int32_t done = fl[2];
    for (EnsHostInst& h : e->inst) h.steps += done;
    left -= done;
    if (fl[0]) {
      // a neighbour row outgrew the list: the call stopped at the start of
      // that step (state re-sorted, nothing else changed); grow and go on
      const int want = std::max(fl[1] + fl[1] / 4 + 8, e->nls + e->nls / 2);
      if ((rc = ens_reserve_list(e, want))) return rc;
      if (++guard > 8) return fail(GCSPH_ECAPACITY, "neighbour list keeps overflowing (%d entries)", fl[1]);
    } else if (left != 0) {
      return fail(GCSPH_ESTATE, "ensemble call stopped %d steps short without an overflow", left);
    }
  }
  return GCSPH_OK;
}

int ens_get(gcsph_ens* e, int32_t slot, int32_t field, double* out_host) {
  if (!e || !out_host) return fail(GCSPH_EINVAL, "null argument");
  size_t pos = 0;
  EnsHostInst* h = find_slot(e, slot, &pos);
  if (!h) return fail(GCSPH_EINVAL, "no instance in slot %d", (int)slot);
  const int D = e->D;
  const int64_t n = h->n;
  int rc;
  const int comps = (field == GCSPH_ENS_X || field == GCSPH_ENS_V) ? D : 1;
  if ((rc = e->OUT.ensure(sizeof(double) * n * comps, e->st))) return rc;
  double* o = e->OUT.as<double>();
  const int b = e->cur;
  const int32_t* id = e->ID[b].as<int32_t>();
  const int nb = nblocks(n, 256);
  switch (field) {
    case GCSPH_ENS_X:
      for (int d = 0; d < D; ++d)
        k_ens_out<<<nb, 256, 0, e->st>>>(n, h->p_off, id, e->X[b][d].as<double>(), nullptr, nullptr, 0, 0.0,
                                          o + (size_t)d * n);
      break;
    case GCSPH_ENS_V:
      for (int d = 0; d < D; ++d)
        k_ens_out<<<nb, 256, 0, e->st>>>(n, h->p_off, id, nullptr, e->V[b][d].as<float>(), nullptr, 1, 0.0,
                                          o + (size_t)d * n);
      break;
    case GCSPH_ENS_RHO:
      k_ens_out<<<nb, 256, 0, e->st>>>(n, h->p_off, id, nullptr, e->DR[b].as<float>(), nullptr, 1, h->prm.rho0, o);
      break;
    case GCSPH_ENS_DRHO:
      k_ens_out<<<nb, 256, 0, e->st>>>(n, h->p_off, id, nullptr, e->DR[b].as<float>(), nullptr, 1, 0.0, o);
      break;
    case GCSPH_ENS_P:
      k_ens_pressure_out<<<nb, 256, 0, e->st>>>(n, h->p_off, id, e->DR[b].as<float>(), e->PT[b].as<int32_t>(),
                                                 e->TAB.as<EnsInst>(), (int)pos, o);
      break;
    case GCSPH_ENS_PTYPE:
      k_ens_out<<<nb, 256, 0, e->st>>>(n, h->p_off, id, nullptr, nullptr, e->PT[b].as<int32_t>(), 2, 0.0, o);
      break;
    default:
      return fail(GCSPH_EINVAL, "unknown ensemble field %d", (int)field);
  }
  GC_LAUNCHED();
  GC_CUDA(cudaMemcpyAsync(out_host, o, sizeof(double) * n * comps, cudaMemcpyDeviceToHost, e->st));
  GC_CUDA(cudaStreamSynchronize(e->st));
  return GCSPH_OK;
}

int ens_info(gcsph_ens* e, int32_t slot, int64_t* n, int64_t* steps, double* etime) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  EnsHostInst* h = find_slot(e, slot);
  if (!h) return fail(GCSPH_EINVAL, "no instance in slot %d", (int)slot);
  if (n) *n = h->n;
  if (steps) *steps = h->steps;
  if (etime) *etime = (double)h->steps * h->prm.dt;
  return GCSPH_OK;
}

int ens_totals(gcsph_ens* e, int32_t* ninst, int64_t* nparticles, int64_t* ncells) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if (ninst) *ninst = (int32_t)e->inst.size();
  if (nparticles) *nparticles = e->N;
  if (ncells) *ncells = e->K;
  return GCSPH_OK;
}

int ens_set_tuning(gcsph_ens* e, int32_t tpb, int32_t graphs) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if (!(tpb == 0 || tpb == 128 || tpb == 256 || tpb == 512)) return fail(GCSPH_EINVAL, "tpb must be 0, 128, 256 or 512");
  e->tpb = tpb;
  e->tpb_fixed = tpb != 0;
  e->tuned_n = 0;
  e->tune_phase = 0;
  e->use_graphs = graphs != 0;
  return GCSPH_OK;
}

int ens_set_list_stride(gcsph_ens* e, int32_t nls) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if (nls < 1 || nls > 4096) return fail(GCSPH_EINVAL, "list stride %d (1..4096)", (int)nls);
  cudaStreamSynchronize(e->st);
  e->NL.release();
  e->nls = 0;
  e->nl_cap = 0;
  e->lists_lost = true;
  return ens_reserve_list(e, nls);
}

int ens_set_skin(gcsph_ens* e, double skin) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if (!(skin >= 0.0 && skin <= 1.0)) return fail(GCSPH_EINVAL, "skin %g (0 .. 1)", skin);
  if (!e->inst.empty()) return fail(GCSPH_ESTATE, "set the skin before adding instances");
  e->skin = skin;
  return GCSPH_OK;
}

int ens_get_skin(gcsph_ens* e, double* skin) {
  if (!e || !skin) return fail(GCSPH_EINVAL, "null argument");
  *skin = e->skin;
  return GCSPH_OK;
}

int ens_set_dpc_bound(gcsph_ens* e, int32_t on) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  e->dpc_bound = on != 0;
  return GCSPH_OK;
}

int ens_get_dpc_bound(gcsph_ens* e, int32_t* on) {
  if (!e || !on) return fail(GCSPH_EINVAL, "null argument");
  *on = e->dpc_bound ? 1 : 0;
  return GCSPH_OK;
}

int ens_list_builds(gcsph_ens* e, int32_t slot, int64_t* builds) {
  if (!e || !builds) return fail(GCSPH_EINVAL, "null argument");
  size_t pos = 0;
  if (!find_slot(e, slot, &pos)) return fail(GCSPH_EINVAL, "no instance in slot %d", (int)slot);
  int32_t v = 0;
  GC_CUDA(cudaMemcpyAsync(&v, e->NREB.as<int32_t>() + pos, sizeof(int32_t), cudaMemcpyDeviceToHost, e->st));
  GC_CUDA(cudaStreamSynchronize(e->st));
  *builds = v;
  return GCSPH_OK;
}

int ens_get_list_stride(gcsph_ens* e, int32_t* nls) {
  if (!e || !nls) return fail(GCSPH_EINVAL, "null argument");
  *nls = e->nls;
  return GCSPH_OK;
}

int ens_set_list_build(gcsph_ens* e, int32_t lanes, int32_t cells_per_block, int32_t depth, int32_t cap) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if (lanes == 0) {
    e->nl_fixed = false;
    if (e->tune_phase > 1) e->tune_phase = 1;
    return GCSPH_OK;
  }
  if (!(lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8)) return fail(GCSPH_EINVAL, "lanes must be 0, 1, 2, 4 or 8");
  if (!(cells_per_block == 0 || cpb_index(cells_per_block) >= 0))
    return fail(GCSPH_EINVAL, "cells per block must be 0, 2, 4, 8 or 16");
  if (depth != 1 && depth != 2) return fail(GCSPH_EINVAL, "staging depth must be 1 or 2");
  if (cap < 0 || (cap > 0 && cap < 32)) return fail(GCSPH_EINVAL, "tile buffer of %d particles (0, or at least 32)", (int)cap);
  e->nl_lanes = lanes;
  e->nl_cpb = cells_per_block;
  e->nl_depth = depth;
  e->nl_cap_fix = cap;
  e->nl_fixed = true;
  return GCSPH_OK;
}

int ens_get_list_build(gcsph_ens* e, int32_t* lanes, int32_t* cells_per_block, int32_t* depth, int32_t* cap) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if (lanes) *lanes = e->nl_lanes;
  if (cells_per_block) *cells_per_block = e->nl_cpb;
  if (depth) *depth = e->nl_depth;
  if (cap) *cap = e->nl_cpb > 0 ? tile_cap(e, e->nl_cpb, e->nl_depth) : 0;
  return GCSPH_OK;
}

int ens_get_tuning(gcsph_ens* e, int32_t* tpb, int32_t* nl_lanes, int64_t* captures, int64_t* replays) {
  if (!e) return fail(GCSPH_EINVAL, "null handle");
  if (tpb) *tpb = e->tpb;
  if (nl_lanes) *nl_lanes = e->nl_lanes;
  if (captures) *captures = e->n_captures;
  if (replays) *replays = e->n_replays;
  return GCSPH_OK;
}

}  // extern "C"
