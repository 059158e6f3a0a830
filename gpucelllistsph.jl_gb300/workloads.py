"""Particle set-ups: dam-break lattices, uniform random clouds, fixture loader.

These stand in for the reference's CSV inputs (src/auxillary.jl:3-11 and
test/input/*.csv) and for the parameter sets of its examples
(README.md:107-123, examples/timesolve3d.jl:15-29).  Coordinates follow the
reference's axis convention: component 2 is vertical (gravity acts on it,
src/sphproblem.jl:10-17); in 3-D component 3 is the tank depth.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SEED = 20261203


@dataclass
class Case:
    """One particle set-up plus the SPHProblem constructor arguments."""
    x: np.ndarray            # (D, N) float64
    rho: np.ndarray          # (N,) float64
    ptype: np.ndarray        # (N,) int32
    dx: float
    h: float
    H: float
    dist: float
    cellsize: tuple
    rho0: float = 1000.0
    m0: float = 0.0
    dt: float = 1e-5
    alpha: float = 0.01
    c0: float = 0.0
    gamma: int = 7
    delta: float = 0.1
    CFL: float = 0.2
    g: float = 9.81
    s: float = 0.0
    extra: dict = field(default_factory=dict)   # mutable fields set after construction
    interior: tuple = None   # per dimension (lo, hi) of the tank interior, for the flow checks

    @property
    def D(self):
        return int(self.x.shape[0])

    @property
    def N(self):
        return int(self.x.shape[1])


def _lattice(lo, hi, dx):
    """Cell-centred lattice coordinates in [lo, hi)."""
    n = int(round((hi - lo) / dx))
    return lo + (np.arange(n) + 0.5) * dx


def dam_break_2d(dx=0.02, fluid=(1.0, 2.0), tank=(4.0, 3.0), layers=3, layer_ptype=None, rho=1000.0,
                 dist_factor=1.0) -> Case:
    """2-D dam break: fluid column fluid[0] x fluid[1] at the left wall of a
    tank[0] x tank[1] tank with `layers` lattice rows of fixed particles on the
    floor and both walls.  layer_ptype[l] is the ptype of boundary row l
    (0 = innermost); default all 0, the fixture convention is (1, 0, 0)."""
    if layer_ptype is None:
        layer_ptype = (0,) * layers
    fx = _lattice(0.0, fluid[0], dx)
    fy = _lattice(0.0, fluid[1], dx)
    FX, FY = np.meshgrid(fx, fy, indexing="ij")
    xs, ys, pts = [FX.ravel()], [FY.ravel()], [np.full(FX.size, 2, np.int32)]
    for l in range(layers):
        off = (l + 0.5) * dx
        # floor row spans the walls' layers too
        bx = np.arange(-(layers - 0.5) * dx, tank[0] + (layers - 0.5) * dx + 0.5 * dx, dx)
        xs.append(bx); ys.append(np.full(bx.size, -off)); pts.append(np.full(bx.size, layer_ptype[l], np.int32))
        wy = _lattice(0.0, tank[1], dx)
        for wx in (-off, tank[0] + off):
            xs.append(np.full(wy.size, wx)); ys.append(wy); pts.append(np.full(wy.size, layer_ptype[l], np.int32))
    x = np.stack([np.concatenate(xs), np.concatenate(ys)]).astype(np.float64)
    ptype = np.concatenate(pts).astype(np.int32)
    h = 1.2 * math.sqrt(2) * dx
    H = 2 * h
    dist = dist_factor * H
    rho0 = 1000.0
    g = 9.81
    return Case(x=np.ascontiguousarray(x), rho=np.full(x.shape[1], float(rho)), ptype=ptype, dx=dx, h=h, H=H,
                dist=dist, cellsize=(dist, dist), rho0=rho0, m0=rho0 * dx * dx, dt=1e-5, alpha=0.01,
                c0=math.sqrt(g * 2) * 20, gamma=7, delta=0.1, CFL=0.2, g=g,
                interior=((0.0, float(tank[0])), (0.0, math.inf)))


def dam_break_3d(dx=0.01, fluid=(1.0, 2.0, 0.5), tank=(4.0, 3.0, 1.0), layers=3, layer_ptype=None, rho=1000.0,
                 dist_factor=1.0, full_physics=True) -> Case:
    """3-D dam break (component 2 vertical): fluid block fluid = (length,
    height, depth) in a tank of (length, height, depth) with `layers` lattice
    layers on the floor and all four walls.  h = sqrt(3 dx^2)
    (examples/timesolve3d.jl:16); full_physics sets ν=0.2, s=0.05, DPC
    l₀=0.005 λ=0.005 pmax=36000, XSPH ε=0.5 (README.md:142-150)."""
    if layer_ptype is None:
        layer_ptype = (1,) + (0,) * (layers - 1)
    fx, fy, fz = (_lattice(0.0, fluid[d], dx) for d in range(3))
    F = np.meshgrid(fx, fy, fz, indexing="ij")
    parts = [np.stack([f.ravel() for f in F])]
    pts = [np.full(F[0].size, 2, np.int32)]
    # boundary: all lattice sites of the enlarged box that are outside the tank
    # interior (x<0 or x>L or z<0 or z>W) or below the floor, within `layers` rows
    L, Ht, W = tank
    bx = (np.arange(-layers, int(round(L / dx)) + layers) + 0.5) * dx
    by = (np.arange(-layers, int(round(Ht / dx))) + 0.5) * dx
    bz = (np.arange(-layers, int(round(W / dx)) + layers) + 0.5) * dx
    BX, BY, BZ = np.meshgrid(bx, by, bz, indexing="ij")
    # layer index = how many rows outside the interior (0 = innermost)
    ox = np.maximum(np.maximum(-BX, BX - L), 0.0)
    oy = np.maximum(-BY, 0.0)
    oz = np.maximum(np.maximum(-BZ, BZ - W), 0.0)
    depth = np.maximum(np.maximum(ox, oy), oz)
    outside = depth > 0
    lay = np.floor(depth / dx + 1e-9).astype(np.int64)
    sel = outside & (lay < layers)
    parts.append(np.stack([BX[sel], BY[sel], BZ[sel]]))
    lp = np.asarray(layer_ptype, np.int32)
    pts.append(lp[lay[sel]])
    x = np.ascontiguousarray(np.concatenate(parts, axis=1).astype(np.float64))
    ptype = np.concatenate(pts).astype(np.int32)
    h = math.sqrt(3 * dx ** 2)
    H = 2 * h
    dist = dist_factor * H
    rho0 = 1000.0
    g = 9.81
    c = Case(x=x, rho=np.full(x.shape[1], float(rho)), ptype=ptype, dx=dx, h=h, H=H, dist=dist,
             cellsize=(dist, dist, dist), rho0=rho0, m0=rho0 * dx * dx * dx, dt=1e-5, alpha=0.01,
             c0=math.sqrt(g * 2) * 20, gamma=7, delta=0.1, CFL=0.2, g=g,
             interior=((0.0, float(L)), (0.0, math.inf), (0.0, float(W))))
    if full_physics:
        c.s = 0.05
        c.extra = dict(nu=0.2, dpc_l0=0.005, dpc_lambda=0.005, dpc_pmax=36000.0, xsph_eps=0.5)
    return c


def uniform_points(N: int, D: int, seed: int = SEED) -> np.ndarray:
    """N uniform points in [0,1)^D, (D, N) float64, numpy PCG64(seed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.ascontiguousarray(rng.random((D, N)))


def load_fixture(path: str) -> Case:
    """Load a compact .npz made from the reference's 2-D CSV fixtures
    (tests/golden/make_golden.py) with the README demo's parameters
    (README.md:107-123)."""
    z = np.load(path)
    x = np.ascontiguousarray(z["x"].astype(np.float64))
    dx = float(z["dx"])
    h = 1.2 * math.sqrt(2) * dx
    H = 2 * h
    rho0 = 1000.0
    g = 9.81
    return Case(x=x, rho=np.ascontiguousarray(z["rho"].astype(np.float64)),
                ptype=np.ascontiguousarray(z["ptype"].astype(np.int32)), dx=dx, h=h, H=H, dist=H,
                cellsize=(H, H), rho0=rho0, m0=rho0 * dx * dx, dt=1e-5, alpha=0.01, c0=math.sqrt(g * 2) * 20,
                gamma=7, delta=0.1, CFL=0.2, g=g)



def _log_uniform(rng, lo, hi):
    return float(math.exp(rng.uniform(math.log(lo), math.log(hi))))


def sized_dam_break_2d(n_fluid: int, aspect: float, dx: float) -> Case:
    """A 2-D dam break whose fluid column holds about n_fluid particles with
    height/width = aspect, in a tank 4x the column's width and 1.5x its
    height (the proportions of the 1.0x2.0 column in the 4.0x3.0 tank).
    c₀ = 10 sqrt(2 g max(height, 4 m)), the reference example's 20 sqrt(2g)
    for columns up to 4 m."""
    nx = max(2, int(round(math.sqrt(n_fluid / aspect))))
    ny = max(2, int(round(n_fluid / nx)))
    W, Hc = nx * dx, ny * dx
    c = dam_break_2d(dx=dx, fluid=(W, Hc), tank=(4.0 * W, 1.5 * Hc))
    c.c0 = 10.0 * math.sqrt(2.0 * c.g * max(Hc, 4.0))
    return c


def sized_dam_break_3d(n_fluid: int, aspect: float, dx: float) -> Case:
    """A 3-D dam break (component 2 vertical) whose fluid block holds about
    n_fluid particles, block (L, aspect L, L/2), tank (4L, 1.5 aspect L, L)."""
    L = dx * (n_fluid / (0.5 * aspect)) ** (1.0 / 3.0)
    L = max(L, 3 * dx)
    block = (L, aspect * L, 0.5 * L)
    c = dam_break_3d(dx=dx, fluid=block, tank=(4.0 * L, 1.5 * aspect * L, L), full_physics=False)
    c.c0 = 10.0 * math.sqrt(2.0 * c.g * max(block[1], 4.0))
    return c


def ensemble_2d(count: int = 256, seed: int = SEED, n_range=(2_000, 200_000), aspect=(0.5, 4.0),
                dx_range=(0.005, 0.02), alpha=(0.005, 0.05), delta=(0.05, 0.2)):
    """The batched-ensemble workload: `count` independent 2-D dam breaks,
    fluid-column particle counts log-uniform in n_range, column aspect, dx,
    α and δ uniform -- numpy PCG64(seed).  Returns a list of (Case, α, δ)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(count):
        n = _log_uniform(rng, *n_range)
        a = float(rng.uniform(*aspect))
        dx = float(rng.uniform(*dx_range))
        al = float(rng.uniform(*alpha))
        de = float(rng.uniform(*delta))
        out.append((sized_dam_break_2d(int(n), a, dx), al, de))
    return out


def serving_requests(count: int, seed: int = SEED, rate: float = 20.0, frac_2d: float = 0.7,
                     n_range=(5_000, 2_000_000), horizon=(0.05, 0.5), horizon_scale: float = 1.0,
                     aspect=(0.5, 4.0), dx_range=(0.005, 0.02)):
    """The serving workload: a Poisson stream (mean `rate` requests/s) of
    dam-break solves, frac_2d of them 2-D, particle counts log-uniform in
    n_range, physical horizons uniform in `horizon` seconds (times
    horizon_scale) at Δt = 1e-5.  Returns [(arrival_s, Case, steps)]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for _ in range(count):
        t += float(rng.exponential(1.0 / rate))
        n = int(_log_uniform(rng, *n_range))
        a = float(rng.uniform(*aspect))
        dx = float(rng.uniform(*dx_range))
        two = bool(rng.uniform() < frac_2d)
        hz = float(rng.uniform(*horizon)) * horizon_scale
        case = sized_dam_break_2d(n, a, dx) if two else sized_dam_break_3d(n, a, dx)
        steps = max(1, int(round(hz / case.dt)))
        out.append((t, case, steps))
    return out


def read_csv_columns(path: str) -> dict:
    """A DualSPHysics/ParaView-style CSV (quoted header, numeric columns) as
    {column name: float64 array} -- the DataFrame the reference reads."""
    import csv
    with open(path, newline="") as f:
        names = next(csv.reader(f))
    data = np.loadtxt(path, delimiter=",", skiprows=1, ndmin=2)
    if data.shape[1] != len(names):
        raise ValueError(f"{path}: {len(names)} header names, {data.shape[1]} columns")
    return {n: np.ascontiguousarray(data[:, i]) for i, n in enumerate(names)}


def loadparticles(fluid_csv: str, boundary_csv: str, fluidcols=("Points:0", "Points:2"),
                  boundarycols=("Points:0", "Points:2")):
    """loadparticles (src/auxillary.jl:3-11): fluid points, then boundary
    points, from the named columns (2-D default: ParaView x and z).  Returns
    (points (D, N) float64, fluid columns, boundary columns)."""
    if len(fluidcols) != len(boundarycols):
        raise ValueError("fluid and boundary column lists differ in length")
    fl = read_csv_columns(fluid_csv)
    bd = read_csv_columns(boundary_csv)
    pts = np.stack([np.concatenate([fl[a], bd[b]]) for a, b in zip(fluidcols, boundarycols)])
    return np.ascontiguousarray(pts), fl, bd


def case_from_csv(fluid_csv: str, boundary_csv: str, dx: float, fluidcols=("Points:0", "Points:2"),
                  boundarycols=("Points:0", "Points:2"), rho_col="Rhop", ptype_col="ptype") -> Case:
    """A Case from the reference's particle CSVs with the README demo's
    parameters (h = 1.2√2 dx in 2-D, √3 dx in 3-D, H = 2h, dist = H): density
    from `rho_col`, ptype from `ptype_col` (fluid rows default to 2 and
    boundary rows to 0 where the column is absent)."""
    x, fl, bd = loadparticles(fluid_csv, boundary_csv, fluidcols, boundarycols)
    D = x.shape[0]
    rho = np.concatenate([fl.get(rho_col, np.full(len(next(iter(fl.values()))), 1000.0)),
                          bd.get(rho_col, np.full(len(next(iter(bd.values()))), 1000.0))])
    nf, nb = len(next(iter(fl.values()))), len(next(iter(bd.values())))
    pt = np.concatenate([fl.get(ptype_col, np.full(nf, 2.0)), bd.get(ptype_col, np.zeros(nb))]).astype(np.int32)
    h = 1.2 * math.sqrt(2) * dx if D == 2 else math.sqrt(3 * dx ** 2)
    H = 2 * h
    rho0, g = 1000.0, 9.81
    return Case(x=x, rho=np.ascontiguousarray(rho, dtype=np.float64), ptype=pt, dx=dx, h=h, H=H, dist=H,
                cellsize=(H,) * D, rho0=rho0, m0=rho0 * dx ** D, dt=1e-5, alpha=0.01, c0=math.sqrt(g * 2) * 20,
                gamma=7, delta=0.1, CFL=0.2, g=g)
