/*
 * gcsph.h -- C ABI of libgcsph.so, the GB300 (sm_103a) hot path of
 * GPUCellListSPH.jl: cell-list binning, the half-stencil pair list, the SPH
 * pair sums and the symplectic step with its CFL reduction.
 *
 * Every pointer named *_dev is a device pointer (a CuPtr from Julia, a
 * torch.Tensor.data_ptr() from Python).  Vector fields are passed as an array
 * of D device pointers held in HOST memory (Julia: Ref(ntuple of CuPtr)), the
 * layout of the reference's NTuple{D, CuArray{T}}.  Particle indices in pair
 * lists are 1-based Int32, (min, max) ordered, exactly as the reference's
 * CuArray{Tuple{Int32,Int32}}.  All calls are synchronous at return (the
 * reference wraps every launch in CUDA.@sync) and report errors by status code
 * plus gcsph_last_error(); nothing traps or throws across the ABI.
 *
 * Citations (file:line) are to the reference package GPUCellListSPH.jl.
 */
#ifndef GCSPH_H
#define GCSPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#define GCSPH_OK 0
#define GCSPH_EINVAL 1     /* bad argument (Julia: error("...")) */
#define GCSPH_ECAPACITY 2  /* caller buffer too small; the needed count is returned */
#define GCSPH_ECUDA 3      /* CUDA runtime error */
#define GCSPH_ENOMEM 4     /* device allocation failed */
#define GCSPH_ESTATE 5     /* call out of order (e.g. pairs requested before a build) */

typedef struct gcl_handle gcl_handle;
typedef struct sph_handle sph_handle;

/* ---------------------------------------------------------------- library */
const char* gcsph_last_error(void);
int gcsph_version(void);
/* number of kernels this library has launched so far (process-wide) */
uint64_t gcsph_launch_count(void);

/* CUDA-event timers per kernel family, recorded on the launching stream
 * (BenchmarkTools / Profile stand-ins, examples/cellist.jl:23-27).  Off by
 * default; names: stage1 stage2 dpc xsph cspm sort pairs state post dt. */
int gcsph_timing_enable(int on);
int gcsph_timing_reset(void);
int gcsph_timing_count(void);
const char* gcsph_timing_name(int32_t id);
int gcsph_timing_get(int32_t id, int64_t* launches, double* total_ms);

/* ---------------------------------------------------------------- cell list */

/* GPUCellList(points, cellsize, dist; MIN, MAX) -- src/celllist.jl:22-88.
 * Freezes the grid (MIN lowered by |(MIN+sqrt(eps))*sqrt(eps)|, CELL =
 * ceil((MAX-MIN)/cs), cs raised to dist) and runs the first build.  x_dev are
 * the D coordinate arrays (the struct's `points`), read on every update and
 * written back by sph_step; they must outlive the handle.  stream may be NULL
 * (legacy default stream). */
int gcl_create(int32_t D, int64_t N, const double* const* x_dev, const double* cellsize, double dist,
               const double* MIN_or_null, const double* MAX_or_null, void* stream, gcl_handle** out);
void gcl_destroy(gcl_handle* h);

/* c.cs, c.offset, c.grid -- src/celllist.jl:1-15 */
int gcl_grid(const gcl_handle* h, double* cs, double* offset, int64_t* cell);

/* update!(c) -- src/celllist.jl:95-134: re-bin every point into the frozen
 * grid, then neib_search! (src/gpukernels_cls.jl:561-587).  *pairsn_out is the
 * pair count (c.pairsn). */
int gcl_update(gcl_handle* h, int64_t* pairsn_out);

/* partialupdate!(c) -- src/celllist.jl:141-145: pair search with the cell
 * membership of the last update and the current coordinates. */
int gcl_partialupdate(gcl_handle* h, int64_t* pairsn_out);

/* neighborlist(c) / neighborlistview(c) -- src/celllist.jl:152-163.  Writes
 * the pair set of the last build as (min,max) 1-based pairs into pairs_dev
 * (2*cap int32).  If the set holds more than cap pairs the first cap are
 * written and GCSPH_ECAPACITY is returned with *pairsn_out = the full count
 * (the reference counts past capacity too, src/gpukernels_cls.jl:333-338).
 * fillzero != 0 zero-fills pairs [pairsn, cap) (src/celllist.jl:112,142). */
int gcl_emit_pairs(gcl_handle* h, int32_t* pairs_dev, int64_t cap, int fillzero, int64_t* pairsn_out);

/* c.cellpnum (Int32[CELL...], column-major) -- src/gpukernels_cls.jl:29-60 */
int gcl_cellpnum(gcl_handle* h, int32_t* cellpnum_dev);

/* мaxpairs(c.cellpnum) -- src/gpukernels_cls.jl:109-286 */
int gcl_maxpairs(gcl_handle* h, int64_t* out);

/* The order inside a cell (by original index) of the binning (no reference
 * counterpart; a tuning knob -- the pair list, its order and every result
 * are the same for every choice).  0 = chosen by the most crowded cell (the
 * default), 1 = the counting sort's in-cell rank (cost: the square of a
 * cell's population), 2 = a stable radix sort (a few passes over the set;
 * sets of more than 65,536 points only). */
int gcl_set_sort(gcl_handle* h, int32_t mode);

/* No counterpart in the reference.  The pair list of GPUCellList(points,
 * cellsize, dist; MIN, MAX) in a single call that allocates no memory, for
 * callers that must not allocate device memory while they run: a host whose
 * own pool already holds the device (a Julia or PyTorch process), a plugin
 * whose framework forbids allocation, a time-critical loop that cannot take
 * cudaMalloc's implicit device synchronisation.  All intermediate arrays sit
 * in one static device array (24 MiB, kept by every GPU that loads the
 * library until the process exits) sized for at most
 * GCSPH_NOALLOC_MAX_POINTS points and GCSPH_NOALLOC_MAX_CELLS grid cells;
 * larger inputs are rejected with GCSPH_EINVAL, and so is a NaN coordinate
 * when MIN/MAX are null (the reference's grid of such a set is an error).
 * Output: the same (min,max) 1-based list, in the same order, that
 * gcl_create + gcl_emit_pairs give; GCSPH_ECAPACITY and the full count when
 * it does not fit in cap.  Every call waits for `stream` before it returns:
 * it reads the bounding box (when MIN/MAX are null) and the pair count back
 * to the host.  Calls share the array: two calls that overlap on the GPU
 * (different streams, threads) race and corrupt each other.
 *
 * CUDA reserves the static array, and loads the kernels of the call, when
 * the library's code is first used on a device (lazy module loading, the
 * CUDA default), and that needs free device memory.  A caller whose own
 * pool is about to take the device's memory calls gcl_pairs_noalloc_init()
 * first, with the device current: it looks up the array's device address
 * and loads every kernel the call launches, once per device.  Otherwise the
 * first gcl_pairs_noalloc call on a device does this set-up itself; make
 * that first call (or the init) before any stream capture. */
#define GCSPH_NOALLOC_MAX_POINTS 262144
#define GCSPH_NOALLOC_MAX_CELLS 1048576
int gcl_pairs_noalloc(int32_t D, int64_t N, const double* const* x_dev, const double* cellsize, double dist,
                      const double* MIN_or_null, const double* MAX_or_null, int32_t* pairs_dev, int64_t cap,
                      int fillzero, int64_t* pairsn_out, void* stream);
/* No counterpart in the reference: the set-up of gcl_pairs_noalloc on the
 * current device (see above); allocates nothing itself, returns 0 or
 * GCSPH_ECUDA. */
int gcl_pairs_noalloc_init(void);

/* ---------------------------------------------------------------- SPH problem */

/* Mutable SPHProblem scalars, src/sphproblem.jl:62-112 (defaults :172-191). */
typedef struct {
  double dx, h, H, rho0, m0, dt, alpha, nu, g, c0, s, delta, CFL, nui, etime;
  double dpc_l0, dpc_pmin, dpc_pmax, dpc_lambda, xsph_eps, bound_D, bound_l;
  int32_t gamma, cspmn;
} gcsph_params;

/* Fields for sph_get_field (src/sphproblem.jl:348-390 getters and the
 * struct's work arrays), always in original particle order. */
enum {
  GCSPH_F_X = 0,      /* get_points        D x N */
  GCSPH_F_RHO = 1,    /* get_density       N */
  GCSPH_F_V = 2,      /* get_velocity      D x N */
  GCSPH_F_P = 3,      /* get_pressure      N */
  GCSPH_F_A = 4,      /* get_acceleration  D x N (∑∂v∂t) */
  GCSPH_F_DRHODT = 5, /* ∑∂ρ∂t             N */
  GCSPH_F_RHOH = 6,   /* ρΔt½              N */
  GCSPH_F_VH = 7,     /* vΔt½              D x N */
  GCSPH_F_XH = 8,     /* xΔt½              D x N */
  GCSPH_F_CDX = 9,    /* cΔx               D x N */
  GCSPH_F_SUMW = 10,  /* get_sumw          N */
  GCSPH_F_SUMGW = 11, /* get_sumgradw      D x N */
  GCSPH_F_BUF2 = 12,  /* buf2 (DPC / XSPH / CSPM sums) D x N */
  GCSPH_F_PTYPE = 13  /* get_ptype         N (int32) */
};

/* SPHProblem(system, dx, h, H, kernel, ρ, ptype, ρ₀, m₀, Δt, α, c₀, γ, δᵩ,
 * CFL; v, g, s) -- src/sphproblem.jl:113-192, WendlandC2 kernel of dimension
 * D.  rho_dev, v_dev (D arrays, or NULL for zeros) and ptype_dev are the
 * caller's arrays; sph_step reads them at entry and writes ρ, v and the
 * cell list's points back before it returns. */
int sph_create(gcl_handle* cl, const gcsph_params* prm, double* rho_dev, double* const* v_dev,
               const int32_t* ptype_dev, sph_handle** out);
void sph_destroy(sph_handle* h);
int sph_set_params(sph_handle* h, const gcsph_params* prm);
int sph_get_params(const sph_handle* h, gcsph_params* prm);

/* Lanes that share one particle in the pair passes (no reference
 * counterpart; a tuning knob).  1 walks each neighbour row serially -- the
 * summation order of a serial scatter over the canonically ordered pair list,
 * bit-identical to the CPU oracle; 2..32 split the row across lanes and
 * combine with a fixed butterfly (FP64 results within 1e-12 of lanes = 1).
 * 0 (default) picks about four neighbours per lane. */
int sph_set_lanes(sph_handle* h, int32_t lanes);

/* Captured calls (no reference counterpart; on by default).  When update! is
 * due after every step (nui <= 0, e.g. dist = H), sph_step runs the whole
 * call -- gather, n steps, scatter, post sums -- as one CUDA graph with one
 * host round trip, instead of one round trip per step.  Results are
 * identical to the per-step loop; a neighbour overflow inside the graph
 * falls back to that loop for the call.  0 turns capture off. */
int sph_set_graphs(sph_handle* h, int32_t on);
/* Δt_stepping's velocity term (src/gpukernels_sph.jl:1316-1326) uses the
 * absolute v·x / (x·x + η²) of each particle, as written.  relative = 1 uses
 * the viscous time-step bound over pairs instead, max |h Δv·Δx / (|Δx|² + η²)|
 * (no reference counterpart; default 0, the reference's formula). */
int sph_set_dt_variant(sph_handle* h, int32_t relative);
/* How many graphs were captured and how many calls ran as a graph replay. */
int sph_graph_stats(const sph_handle* h, int64_t* captures, int64_t* replays);

/* stepsolve!(prob, n; timestepping, timelims) -- src/sphproblem.jl:204-345.
 * Returns (updaten, maxcΔxout) through the out pointers. */
int sph_step(sph_handle* h, int32_t n, int timestepping, double tmin, double tmax, int64_t* updaten,
             double* maxcdx);

/* copy one field (enum above) into a caller device buffer */
int sph_get_field(sph_handle* h, int32_t field, void* dst_dev);

/* ---------------------------------------------------------------- pair kernels
 * The reference's exported kernel functions, driven by a caller pair list
 * (1-based (i,j), rows with i == 0 skipped) over caller device arrays, one
 * thread per pair with FP64 atomics like the reference.  x/v/∇W/a/buf are
 * arrays of D device pointers (host memory).  stream may be NULL. */

/* sphW!(W, pairs, points, H⁻¹, kernel) -- src/gpukernels_sph.jl:75-100 */
int gcsph_sphW(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* x_dev,
               double Hinv, double* W_dev, void* stream);
/* sph∇W!(∇W, pairs, points, H⁻¹, kernel) -- :186-213 */
int gcsph_sphgradW(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* x_dev,
                   double Hinv, double* const* gW_dev, void* stream);
/* sph∑W!(∑W, pairs, points, kernel, H⁻¹, ptype) -- :129-156 (adds) */
int gcsph_sphsumW(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* x_dev,
                  double Hinv, const int32_t* ptype_dev, double* sumW_dev, void* stream);
/* sph∑∇W!(∑∇W, pairs, points, kernel, H⁻¹, ptype) -- :322-359 (adds) */
int gcsph_sphsumgradW(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* x_dev,
                      double Hinv, const int32_t* ptype_dev, double* const* sumgW_dev, void* stream);
/* ∂ρ∂tDDT!(∑∂ρ∂t, pairs, ∇W, ρ, v, points, h, m₀, ρ₀, c₀, γ, g, δᵩ, ptype) -- :542-631 (zeroes first) */
int gcsph_drhodt_ddt(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* gW_dev,
                     const double* rho_dev, const double* const* v_dev, const double* const* x_dev, double h,
                     double m0, double rho0, double c0, int32_t gamma, double g, double delta,
                     const int32_t* ptype_dev, double* drhodt_dev, void* stream);
/* pressure!(P, ρ, c₀, γ, ρ₀, ptype) -- :710-727 */
int gcsph_pressure(int64_t N, const double* rho_dev, double c0, int32_t gamma, double rho0,
                   const int32_t* ptype_dev, double* P_dev, void* stream);
/* ∂v∂t!(∑∂v∂t, ∇W, P, pairs, m₀, ρ, ptype) -- :740-776 (adds) */
int gcsph_dvdt(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* gW_dev,
               const double* P_dev, double m0, const double* rho_dev, const int32_t* ptype_dev,
               double* const* a_dev, void* stream);
/* ∂v∂t_av!(∑∂v∂t, ∇W, pairs, points, h, ρ, α, v, c₀, m₀, ptype) -- :852-901 (adds) */
int gcsph_dvdt_av(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* gW_dev,
                  const double* const* x_dev, double h, const double* rho_dev, double alpha,
                  const double* const* v_dev, double c0, double m0, const int32_t* ptype_dev,
                  double* const* a_dev, void* stream);
/* ∂v∂t_visc!(∑∂v∂t, ∇W, v, ρ, points, pairs, h, m₀, 𝜈, ptype) -- :952-991 (adds) */
int gcsph_dvdt_visc(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* gW_dev,
                    const double* const* v_dev, const double* rho_dev, const double* const* x_dev, double h,
                    double m0, double nu, const int32_t* ptype_dev, double* const* a_dev, void* stream);
/* ∂v∂t_addgrav!(∑∂v∂t, gravvec(g, dim)) -- :1031-1051, src/sphproblem.jl:10-17 */
int gcsph_addgrav(int32_t D, int64_t N, double g, double* const* a_dev, void* stream);
/* fbmolforce!(∑∂v∂t, pairs, points, d, r₀, ptype) -- :1875-1913 (adds) */
int gcsph_fbmolforce(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* x_dev,
                     double d, double r0, const int32_t* ptype_dev, double* const* a_dev, void* stream);
/* ∂v∂tpF!(∑∂v∂t, pairs, points, s, h, m₀, ptype) -- :1373-1409 (adds) */
int gcsph_dvdt_pF(int32_t D, int64_t N, int64_t P, const int32_t* pairs_dev, const double* const* x_dev,
                  double s, double h, double m0, const int32_t* ptype_dev, double* const* a_dev, void* stream);
/* update_ρp∂ρ∂tΔt!(ρ, ∑∂ρ∂t, Δt, ρ₀, ptype) -- :1078-1096 */
int gcsph_update_rho(int64_t N, double* rho_dev, const double* drhodt_dev, double dt, double rho0,
                     const int32_t* ptype_dev, void* stream);
/* update_vp∂v∂tΔt!(v, ∑∂v∂t, Δt, ptype) -- :1107-1127 */
int gcsph_update_v(int32_t D, int64_t N, double* const* v_dev, const double* const* a_dev, double dt,
                   const int32_t* ptype_dev, void* stream);
/* update_xpvΔt!(x, v, Δt) -- :1150-1169 */
int gcsph_update_x(int32_t D, int64_t N, double* const* x_dev, const double* const* v_dev, double dt,
                   void* stream);
/* symplectic_update!(ρ, ρΔt½, v, vΔt½, x, xΔt½, ∑∂ρ∂t, ∑∂v∂t, Δt, cΔx, ρ₀, ptype) -- :1193-1245 */
int gcsph_symplectic(int32_t D, int64_t N, double* rho_dev, double* rhoh_dev, double* const* v_dev,
                     double* const* vh_dev, double* const* x_dev, double* const* xh_dev,
                     const double* drhodt_dev, const double* const* a_dev, double dt, double* const* cdx_dev,
                     double rho0, const int32_t* ptype_dev, void* stream);
/* dpcreg!(∑Δvdpc, v, ρ, P, pairs, points, kernel, l₀, Pmin, Pmax, Δt, λ, dpckernlim, ptype) -- :1485-1553 (zeroes first) */
int gcsph_dpcreg(int32_t D, int64_t N, int64_t P, double* const* buf_dev, const double* const* v_dev,
                 const double* rho_dev, const double* P_dev, const int32_t* pairs_dev, const double* const* x_dev,
                 double l0, double Pmin, double Pmax, double dt, double lambda, double dpckernlim,
                 const int32_t* ptype_dev, void* stream);
/* update_dpcreg!(v, x, ∑Δvdpc, Δt, ptype) -- :1607-1632 */
int gcsph_update_dpcreg(int32_t D, int64_t N, double* const* v_dev, double* const* x_dev,
                        const double* const* buf_dev, double dt, const int32_t* ptype_dev, void* stream);
/* xsphcorr!(∑Δvxsph, pairs, W, ρ, v, m₀, 𝜀, ptype) -- :1745-1779 (zeroes first) */
int gcsph_xsphcorr(int32_t D, int64_t N, int64_t P, double* const* buf_dev, const int32_t* pairs_dev,
                   const double* W_dev, const double* rho_dev, const double* const* v_dev, double m0, double eps,
                   const int32_t* ptype_dev, void* stream);
/* update_xsphcorr!(x, ∑Δvxsph, Δt, ptype) -- :1817-1838 */
int gcsph_update_xsph(int32_t D, int64_t N, double* const* x_dev, const double* const* buf_dev, double dt,
                      const int32_t* ptype_dev, void* stream);
/* cspmcorr!(∑ρcspm, W, ρ, m₀, pairs, ptype) -- :1673-1719 (zeroes buf first; updates ρ) */
int gcsph_cspmcorr(int32_t D, int64_t N, int64_t P, double* const* buf_dev, const double* W_dev,
                   double* rho_dev, double m0, const int32_t* pairs_dev, const int32_t* ptype_dev, void* stream);
/* Δt_stepping(buf, a, v, points, c₀, h, CFL, timelims) -- :1293-1353; *dt_out is the new Δt */
int gcsph_dt_stepping(int32_t D, int64_t N, const double* const* a_dev, const double* const* v_dev,
                      const double* const* x_dev, double c0, double h, double CFL, double tmin, double tmax,
                      double* dt_out, void* stream);
/* dpckernlim = find_zero(x -> 1 - 𝒲(k, x, 1), 0.5) -- src/sphproblem.jl:218 (host scalar) */
double gcsph_dpckernlim(int32_t D);

/* ------------------------------------------------------------------------
 * Batched FP32 ensemble (no reference counterpart: the reference steps one
 * SPHProblem at a time).  Each step re-sorts all instances into cell order
 * and builds one neighbour list (cell walk, r < H), which every pair pass of
 * the step then walks.  Many independent instances -- each its own particle
 * set, parameters, frozen cell grid (cell edge = H) and fixed Δt -- advance
 * together, one launch per pass over all of them.  Pair arithmetic and
 * per-particle sums in FP32 (Kahan), density held as ρ - ρ₀, positions in
 * FP64.  The physics per step is that of sph_step with dist = H: ∂ρ∂tDDT!,
 * ∂v∂t!, ∂v∂t_av!, ∂v∂t_visc! (ν > 0), gravity!, fbmolforce!, ∂v∂tpF! (s > 0),
 * the half-step predictors, symplectic_update!, dpcreg! (dpc_l0 > 0),
 * xsphcorr! (xsph_eps > 0) and cspmcorr! every cspmn steps (counted from the
 * instance's admission, as within one stepsolve!).  An instance's results do
 * not depend on which other instances share the ensemble (bit-identical).
 * Host arrays in ens_add / ens_get are HOST pointers, D-major (x[d*n + i]).
 * ------------------------------------------------------------------------ */
typedef struct gcsph_ens gcsph_ens;
typedef struct {
  double dx, h, H, rho0, m0, dt, alpha, nu, g, c0, s, delta;
  double bound_D, bound_l;           /* stage-2 fbmolforce constants (stage 1: 0.4, 2dx) */
  double grid_min[3], grid_max[3];   /* frozen cell grid; points outside clamp to edge cells */
  double dpc_l0, dpc_pmin, dpc_pmax, dpc_lambda;  /* dpcreg! when dpc_l0 > 0 */
  double xsph_eps;                   /* xsphcorr! when > 0 */
  int32_t gamma;
  int32_t cspmn;                     /* cspmcorr! every cspmn steps since admission (0: never) */
} gcsph_ens_params;

enum { GCSPH_ENS_X = 0, GCSPH_ENS_V = 1, GCSPH_ENS_RHO = 2, GCSPH_ENS_P = 3, GCSPH_ENS_PTYPE = 4, GCSPH_ENS_DRHO = 5 };

int ens_create(int32_t D, void* stream, gcsph_ens** out);
void ens_destroy(gcsph_ens* e);
/* device bytes one particle needs (admission by free HBM) */
int ens_bytes_per_particle(int32_t D, int64_t* bytes);
/* admit an instance of n particles; v may be NULL (at rest); returns its slot */
int ens_add(gcsph_ens* e, int64_t n, const double* x, const double* v, const double* rho, const int32_t* ptype,
            const gcsph_ens_params* p, int32_t* slot);
int ens_remove(gcsph_ens* e, int32_t slot);
/* n steps of every instance (a captured graph per n; the first steps after a
 * layout change may time three block sizes -- ordinary steps all the same) */
int ens_step(gcsph_ens* e, int32_t n);
/* the stream of the ensemble's later calls (NULL: the legacy default
 * stream); waits for the work of the current one first */
int ens_set_stream(gcsph_ens* e, void* stream);
/* one field of one instance, in its original particle order, as double */
int ens_get(gcsph_ens* e, int32_t slot, int32_t field, double* out_host);
int ens_info(gcsph_ens* e, int32_t slot, int64_t* n, int64_t* steps, double* etime);
int ens_totals(gcsph_ens* e, int32_t* ninst, int64_t* nparticles, int64_t* ncells);
/* tpb 0 = autotune: the pair passes' block size (128/256/512), then the
 * lanes per particle of the neighbour-list build (1/2/4/8), then its tiling
 * (ens_set_list_build) -- the results do not depend on any of them.  graphs
 * 0 = one launch sequence per step. */
int ens_set_tuning(gcsph_ens* e, int32_t tpb, int32_t graphs);
int ens_get_tuning(gcsph_ens* e, int32_t* tpb, int32_t* nl_lanes, int64_t* captures, int64_t* replays);
/* The neighbour-list build (no counterpart in the reference, which has no
 * ensembles; its pair search is src/gpukernels_cls.jl:293-587).  lanes 0 =
 * autotuned.  Otherwise lanes (1/2/4/8) per particle; cells_per_block 0 = one
 * thread group per particle, 2/4/8/16 = a block per tile of that many cells
 * of one x-row, with the tile's neighbourhood staged in shared memory, depth
 * 1 or 2 tiles at a time (2: the next tile is copied while this one is
 * tested); cap = particles a tile buffer holds (0: sized from (H/dx)^D; a tile
 * that does not fit reads global memory).  The list, and every result, is the
 * same for every choice. */
int ens_set_list_build(gcsph_ens* e, int32_t lanes, int32_t cells_per_block, int32_t depth, int32_t cap);
/* The list's skin (no counterpart in the reference, whose update! rebuilds
 * when max |cΔx| > 0.9 (dist - H), src/sphproblem.jl:222-232): cells and list
 * radius of H (1 + skin); an instance rebuilds its cells and list when one of
 * its particles has moved about skin H / 2 since the last build, and every
 * pass keeps only the pairs with r < H at the step's positions.  Default 0.05
 * in 2-D, 0.025 in 3-D; 0 rebuilds at every step.  Set before the first
 * ens_add. */
int ens_set_skin(gcsph_ens* e, double skin);
int ens_get_skin(gcsph_ens* e, double* skin);
/* list builds of one instance so far */
int ens_list_builds(gcsph_ens* e, int32_t slot, int64_t* builds);
/* dpcreg!'s row bound (on by default; no counterpart in the reference, whose
 * dpcreg!, src/gpukernels_sph.jl:1500-1553, evaluates every pair): a row whose
 * smallest separation at the step's start, less the particle's move and the
 * largest move in its instance, clears l0 has no pair within l0 after the
 * step, and its scan is skipped.  Results are the same with the bound on and
 * off; off scans every row. */
int ens_set_dpc_bound(gcsph_ens* e, int32_t on);
int ens_get_dpc_bound(gcsph_ens* e, int32_t* on);
int ens_get_list_build(gcsph_ens* e, int32_t* lanes, int32_t* cells_per_block, int32_t* depth, int32_t* cap);
/* Entries per particle in the step's neighbour list (default 64 in 2-D, 256
 * in 3-D; it grows by itself when a row outgrows it, repeating the steps
 * that had not completed). */
int ens_set_list_stride(gcsph_ens* e, int32_t nls);
int ens_get_list_stride(gcsph_ens* e, int32_t* nls);

/* ---------------------------------------------------------------------------
 * Serving: continuous batching of dam-break solves over the ensembles (no
 * counterpart in the reference, which solves one SPHProblem per call,
 * src/sphproblem.jl:204-345, :420-511).  Submitted requests are admitted
 * once they have arrived and the device has room (n x bytes per particle x 2
 * within 1 - reserve of the free memory) -- in arrival order, or smallest
 * work first within caps (srv_set_policy) -- advance together in chunks of at
 * most `chunk` steps cut at the nearest horizon, and release their slot at
 * their horizon after the fields in `fields` (bit f = GCSPH_ENS field f) are
 * read back.  Times are seconds since srv_create.
 * ------------------------------------------------------------------------ */
typedef struct gcsph_srv gcsph_srv;
/* The scheduler's view of the ensembles, the free memory and the clock.  NULL
 * in srv_create selects the library's own (ens_*, cudaMemGetInfo, a steady
 * clock); a caller's table drives the same scheduling (e.g. host-side tests
 * against a fake ensemble).  Callbacks return 0 or an error code. */
typedef struct gcsph_srv_backend {
  void* ctx;
  int (*add)(void* ctx, int32_t D, int32_t rid, int32_t* slot);
  int (*remove)(void* ctx, int32_t D, int32_t slot);
  int (*step)(void* ctx, int32_t D, int32_t n);
  int (*harvest)(void* ctx, int32_t D, int32_t slot, int32_t rid); /* read results before the remove */
  int64_t (*free_bytes)(void* ctx);
  int64_t (*bytes_per_particle)(void* ctx, int32_t D);
  double (*now)(void* ctx); /* NULL: the library's steady clock */
} gcsph_srv_backend;
typedef struct gcsph_srv_stats {
  int32_t requests, completed;
  int64_t particle_steps;
  double wall_s; /* time of the last completion */
  double p50_s, p99_s, mean_s; /* time to horizon (arrival to results on the host); NaN before any */
} gcsph_srv_stats;
enum { GCSPH_SRV_QUEUED = 0, GCSPH_SRV_RUNNING = 1, GCSPH_SRV_DONE = 2 };
/* admission policies: arrival order (the default), or smallest work
 * (particles x steps) first while a dimension's particles in flight stay
 * within its cap (0: no cap; an idle dimension admits any solve) */
enum { GCSPH_SRV_ARRIVAL = 0, GCSPH_SRV_SHORTEST = 1 };

int srv_create(void* stream, int32_t chunk, double reserve, uint32_t fields, const gcsph_srv_backend* backend,
               gcsph_srv** out);
void srv_destroy(gcsph_srv* s);
/* a request: its particles (host arrays as for ens_add; with a caller's
 * backend they may be NULL), its horizon in steps and its arrival time
 * (negative: now); *rid numbers the requests from 0 */
int srv_submit(gcsph_srv* s, int32_t D, int64_t n, const double* x, const double* v, const double* rho,
               const int32_t* ptype, const gcsph_ens_params* p, int64_t steps, double arrival, int32_t* rid);
/* the admission policy and, for GCSPH_SRV_SHORTEST, the particles in flight
 * per dimension and the longest wait: a solve that has waited max_wait
 * seconds is admitted as soon as it fits, cap or not (0: never), so that a
 * stream of small solves cannot hold a large one back for ever */
int srv_set_policy(gcsph_srv* s, int32_t policy, int64_t cap2d, int64_t cap3d, double max_wait);
int srv_get_policy(gcsph_srv* s, int32_t* policy, int64_t* cap2d, int64_t* cap3d, double* max_wait);
/* one round (admissions, one chunk per ensemble, releases) */
int srv_progress(gcsph_srv* s, int32_t* running, int32_t* queued);
/* rounds until every submitted request has reached its horizon, waiting for
 * arrivals; GCSPH_ECAPACITY if an arrived request cannot fit on an idle device */
int srv_run(gcsph_srv* s);
int srv_request(gcsph_srv* s, int32_t rid, int32_t* state, double* arrival, double* admitted, double* done);
/* a finished request's field, in its original particle order (library backend) */
int srv_result(gcsph_srv* s, int32_t rid, int32_t field, double* out_host);
int srv_stats(gcsph_srv* s, gcsph_srv_stats* st);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* GCSPH_H */
