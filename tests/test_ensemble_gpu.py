"""Batched FP32 ensemble against the FP64 oracle, and its isolation contract.

Tolerance (the FP32 contract): after 100 steps, relative L2 error in ρ and v
against the FP64 oracle at most 1e-4; the displacement from the start within
1e-4 relative L2 as well.  An instance's results are bit-identical alone and
in a mix, whatever joined or left the ensemble, and whatever launch shape or
capture mode ran it.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_l2(got, want):
    got = np.asarray(got, dtype=np.float64).ravel()
    want = np.asarray(want, dtype=np.float64).ravel()
    n = np.linalg.norm(want)
    return np.linalg.norm(got - want) / n if n > 0 else np.linalg.norm(got - want)


def oracle_run(orc, case, n, nu=0.0, s=0.0):
    p = orc.default_params(case.dx, case.h, case.H, case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma,
                           case.delta, case.CFL, case.dist, g=case.g, s=s)
    p.nu = nu
    ref = orc.OracleSystem(case.x, case.cellsize, case.dist, case.rho, case.ptype, p)
    ref.stepsolve(n)
    return ref


def errors(ens, slot, ref, case):
    x = ens.get(slot, "x")
    return {
        "rho": rel_l2(ens.get(slot, "rho"), ref.get("rho")),
        "drho": rel_l2(ens.get(slot, "rho") - case.rho0, ref.get("rho") - case.rho0),
        "v": rel_l2(ens.get(slot, "v"), ref.get("v")),
        "disp": rel_l2(x - case.x, ref.get("x") - case.x),
    }


def test_fp32_dam_break_2d_c1_against_fp64(gpu_pkg, orc):
    """The plain FP64 configuration's dam break (dx = 0.02), 100 steps."""
    case = gpu_pkg.workloads.dam_break_2d()
    ens = gpu_pkg.Ensemble(2)
    slot = ens.add(gpu_pkg.spec_from_case(case))
    ens.step(100)
    assert ens.info(slot)["steps"] == 100
    ref = oracle_run(orc, case, 100)
    err = errors(ens, slot, ref, case)
    print("fp32 vs fp64, 2-D dam break dx=0.02, 100 steps:", err)
    assert err["rho"] <= TOL and err["v"] <= TOL and err["disp"] <= TOL, err
    assert np.array_equal(ens.get(slot, "ptype"), case.ptype)


def test_fp32_3d_viscous_surface_tension_against_fp64(gpu_pkg, orc):
    """A small 3-D block with ν and surface tension on, 100 steps."""
    case = gpu_pkg.workloads.dam_break_3d(dx=0.04, fluid=(0.4, 0.6, 0.2), tank=(0.8, 0.8, 0.3),
                                          full_physics=False)
    spec = gpu_pkg.spec_from_case(case)
    spec.nu, spec.s = 0.2, 0.05
    ens = gpu_pkg.Ensemble(3)
    slot = ens.add(spec)
    ens.step(100)
    ref = oracle_run(orc, case, 100, nu=0.2, s=0.05)
    err = errors(ens, slot, ref, case)
    print("fp32 vs fp64, 3-D block, 100 steps:", err)
    assert err["rho"] <= TOL and err["v"] <= TOL and err["disp"] <= TOL, err


def _oracle_full(orc, case, n, v):
    p = orc.default_params(case.dx, case.h, case.H, case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma,
                           case.delta, case.CFL, case.dist, g=case.g, s=case.s)
    for k, val in case.extra.items():
        setattr(p, k, val)
    ref = orc.OracleSystem(case.x, case.cellsize, case.dist, case.rho, case.ptype, p, v=v)
    ref.stepsolve(n)
    return ref


def _moving(case, seed=17, amp=0.05):
    """Random fluid velocities, so that DPC's branch on the sign of Δv·Δx is
    not decided by rounding noise (lattice pairs at rest)."""
    rng = np.random.default_rng(seed)
    v = rng.uniform(-amp, amp, case.x.shape)
    v[:, case.ptype <= 1] = 0.0
    return np.ascontiguousarray(v)


@pytest.mark.parametrize("D", [2, 3])
def test_fp32_full_physics_against_fp64(gpu_pkg, orc, D):
    """ν, surface tension, DPC, XSPH and CSPM on (dpcreg!/xsphcorr! move x and
    v but not the half-step bases, as in the reference)."""
    w = gpu_pkg.workloads
    if D == 2:
        case = w.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0), layer_ptype=(1, 0, 0))
        case.s = 0.05
        case.extra = dict(nu=0.2, dpc_l0=case.dx * 0.7, dpc_lambda=0.005, dpc_pmax=36000.0, xsph_eps=0.5, cspmn=7)
        n = 60
    else:
        case = w.dam_break_3d(dx=0.05, fluid=(0.3, 0.4, 0.2), tank=(0.6, 0.6, 0.3))
        case.extra = dict(case.extra, dpc_l0=0.03)
        n = 40
    v = _moving(case)
    spec = gpu_pkg.spec_from_case(case)
    spec.v = v
    assert spec.dpc_l0 > 0 and spec.xsph_eps > 0 and spec.nu > 0 and spec.s > 0
    ens = gpu_pkg.Ensemble(D)
    slot = ens.add(spec)
    ens.step(n)
    ref = _oracle_full(orc, case, n, v)
    err = errors(ens, slot, ref, case)
    print(f"fp32 vs fp64, full physics {D}-D, {n} steps:", err)
    assert err["rho"] <= TOL and err["v"] <= TOL and err["disp"] <= TOL, err


def _min_sep(x, rows):
    """Smallest distance from each particle in `rows` to another (brute force)."""
    idx = np.flatnonzero(rows)
    d2 = ((x[:, idx, None] - x[:, None, :]) ** 2).sum(axis=0)
    d2[np.arange(idx.size), idx] = np.inf
    return np.sqrt(d2.min(axis=1))


@pytest.mark.parametrize("D", [2, 3])
def test_dpc_row_bound_changes_nothing(gpu_pkg, D):
    """dpcreg!'s row bound skips only rows with no pair within l0 after the
    step.  Fluid jittered by up to 0.25 dx with l0 = 0.7 dx gives rows with
    pairs within l0 and rows without; every field is bit-identical with the
    bound on and off, and DPC does move the particles (l0 = 0 differs)."""
    w = gpu_pkg.workloads
    if D == 2:
        case = w.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0))
        n = 40
    else:
        case = w.dam_break_3d(dx=0.05, fluid=(0.3, 0.4, 0.2), tank=(0.6, 0.6, 0.3))
        n = 30
    rng = np.random.default_rng(5)
    fl = case.ptype > 1
    case.x = case.x.copy()
    case.x[:, fl] += rng.uniform(-0.25 * case.dx, 0.25 * case.dx, (D, int(fl.sum())))
    l0 = 0.7 * case.dx
    near = _min_sep(case.x, fl) < l0  # about a quarter of the fluid rows at the start
    assert 0.05 < near.mean() < 0.9, near.mean()
    runs = {}
    for name, bound, dpc in (("on", True, l0), ("off", False, l0), ("nodpc", True, 0.0)):
        spec = gpu_pkg.spec_from_case(case)
        spec.v = _moving(case)
        spec.dpc_l0, spec.dpc_lambda, spec.dpc_pmax = dpc, 0.005, 36000.0
        ens = gpu_pkg.Ensemble(D)
        ens.set_dpc_bound(bound)
        assert ens.dpc_bound() == bound
        slot = ens.add(spec)
        ens.step(n)
        runs[name] = {f: ens.get(slot, f) for f in FIELDS}
        ens.close()
    for f in FIELDS:
        assert np.array_equal(runs["on"][f], runs["off"][f]), f
    assert not np.array_equal(runs["on"]["x"], runs["nodpc"]["x"])


def _specs(pkg):
    w = pkg.workloads
    a = pkg.spec_from_case(w.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0)))
    b = pkg.spec_from_case(w.dam_break_2d(dx=0.03, fluid=(0.3, 0.9), tank=(1.0, 1.2)), alpha=0.03, delta=0.15)
    c = pkg.spec_from_case(w.dam_break_2d(dx=0.05, fluid=(1.0, 0.5), tank=(2.0, 1.0)), dt=2e-5)
    d = pkg.spec_from_case(w.dam_break_2d(dx=0.025, fluid=(0.5, 0.5), tank=(0.8, 0.8)))
    return a, b, c, d


FIELDS = ("x", "v", "rho", "P", "ptype")


def test_same_alone_and_in_the_mix(gpu_pkg):
    a, b, c, d = _specs(gpu_pkg)
    alone = gpu_pkg.Ensemble(2)
    sa = alone.add(a)
    alone.step(30)
    alone.step(20)
    mix = gpu_pkg.Ensemble(2)
    mix.add(b)
    sm = mix.add(a)
    sc = mix.add(c)
    mix.step(30)
    mix.remove(sc)          # one leaves ...
    mix.add(d)              # ... another joins
    mix.step(20)
    assert mix.info(sm)["steps"] == 50
    for f in FIELDS:
        assert np.array_equal(alone.get(sa, f), mix.get(sm, f)), f


def test_late_admission_matches_a_fresh_run(gpu_pkg):
    a, b, c, _ = _specs(gpu_pkg)
    fresh = gpu_pkg.Ensemble(2)
    sf = fresh.add(c)
    fresh.step(25)
    busy = gpu_pkg.Ensemble(2)
    busy.add(a)
    busy.add(b)
    busy.step(40)
    sl = busy.add(c)
    busy.step(25)
    assert busy.info(sl)["steps"] == 25
    for f in FIELDS:
        assert np.array_equal(fresh.get(sf, f), busy.get(sl, f)), f


@pytest.mark.parametrize("tpb,graphs", [(128, True), (512, False), (0, True)])
def test_launch_shape_and_capture_do_not_change_results(gpu_pkg, tpb, graphs):
    a, b, _, _ = _specs(gpu_pkg)
    ref = gpu_pkg.Ensemble(2)
    ref.set_tuning(256, False)
    r1, r2 = ref.add(a), ref.add(b)
    ref.step(12)
    ens = gpu_pkg.Ensemble(2)
    ens.set_tuning(tpb, graphs)
    e1, e2 = ens.add(a), ens.add(b)
    ens.step(5)
    ens.step(16)
    ref.step(9)
    for f in FIELDS:
        assert np.array_equal(ref.get(r1, f), ens.get(e1, f)), f
        assert np.array_equal(ref.get(r2, f), ens.get(e2, f)), f
    t = ens.tuning()
    if graphs:
        assert t["replays"] >= 1
    if tpb:
        assert t["tpb"] == tpb
    else:
        assert t["tpb"] in (128, 256, 512) and t["list_lanes"] in (1, 2, 4, 8)


@pytest.mark.parametrize("graphs,build", [(True, None), (False, None), (True, (2, 8, 2, 0)), (False, (1, 4, 1, 0))])
def test_neighbour_list_overflow_grows_and_repeats(gpu_pkg, graphs, build):
    """A list stride far too small: the call stops at the first step whose
    rows do not fit, the stride grows and the remaining steps run -- the
    result is bit-identical to a run that never overflowed, with either list
    build."""
    a, b, _, _ = _specs(gpu_pkg)
    ref = gpu_pkg.Ensemble(2)
    r1, r2 = ref.add(a), ref.add(b)
    ref.step(9)
    ens = gpu_pkg.Ensemble(2)
    ens.set_tuning(256, graphs)
    if build:
        ens.set_list_build(*build)
    e1, e2 = ens.add(a), ens.add(b)
    ens.set_list_stride(4)
    ens.step(9)
    assert ens.list_stride() > 4
    assert ens.info(e1)["steps"] == 9
    for f in FIELDS:
        assert np.array_equal(ref.get(r1, f), ens.get(e1, f)), f
        assert np.array_equal(ref.get(r2, f), ens.get(e2, f)), f


def _specs3(pkg):
    w = pkg.workloads
    a = pkg.spec_from_case(w.dam_break_3d(dx=0.05, fluid=(0.3, 0.4, 0.2), tank=(0.6, 0.6, 0.3), full_physics=False))
    b = pkg.spec_from_case(w.dam_break_3d(dx=0.06, fluid=(0.4, 0.3, 0.3), tank=(0.9, 0.5, 0.4), full_physics=False),
                           alpha=0.03)
    return a, b


@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("lanes,cpb,depth,cap", [(1, 4, 1, 0), (2, 8, 2, 0), (4, 16, 1, 0), (8, 2, 2, 0),
                                                  (2, 4, 1, 32), (1, 8, 2, 64)])
def test_list_build_variants_give_the_same_results(gpu_pkg, D, lanes, cpb, depth, cap):
    """Every neighbour-list build -- a thread group per particle, or tiles of
    cells with their neighbourhood staged in shared memory, one or two tiles
    at a time, and tiles too big for a small buffer (read from global memory)
    -- gives the same list in the same order, so the same results bit for bit,
    over several instances with different grids."""
    specs = _specs(gpu_pkg)[:3] if D == 2 else _specs3(gpu_pkg)
    ref = gpu_pkg.Ensemble(D)
    ref.set_tuning(256, False)
    ref.set_list_build(4, 0, 1, 0)
    rs = [ref.add(s) for s in specs]
    ref.step(12)
    ens = gpu_pkg.Ensemble(D)
    ens.set_tuning(256, True)
    ens.set_list_build(lanes, cpb, depth, cap)
    es = [ens.add(s) for s in specs]
    ens.step(5)
    ens.step(7)
    for r, e in zip(rs, es):
        for f in FIELDS:
            assert np.array_equal(ref.get(r, f), ens.get(e, f)), (f, r)
    t = ens.tuning()
    assert (t["list_lanes"], t["cells_per_block"], t["staging_depth"]) == (lanes, cpb, depth)
    if cap:
        assert t["tile_capacity"] == cap
    else:
        assert t["tile_capacity"] >= 32


def test_autotuner_tries_the_tiled_list_build(gpu_pkg):
    """With enough steps in a call, the tuner runs all three phases (block
    size, list lanes, list tiling) and the results match a run that was
    never tuned."""
    a, b, c, _ = _specs(gpu_pkg)
    ens = gpu_pkg.Ensemble(2)
    es = [ens.add(s) for s in (a, b, c)]
    ens.step(30)
    t = ens.tuning()
    assert t["tpb"] in (128, 256, 512) and t["list_lanes"] in (1, 2, 4, 8)
    assert t["cells_per_block"] in (0, 4, 8, 16) and t["staging_depth"] in (1, 2)
    ref = gpu_pkg.Ensemble(2)
    ref.set_tuning(256, False)
    rs = [ref.add(s) for s in (a, b, c)]
    ref.step(30)
    for r, e in zip(rs, es):
        for f in FIELDS:
            assert np.array_equal(ref.get(r, f), ens.get(e, f)), f


def _fast_spec(pkg, case, amp, seed=11):
    spec = pkg.spec_from_case(case)
    spec.v = _moving(case, seed=seed, amp=amp)
    return spec


@pytest.mark.parametrize("skin", [0.0, 0.02, 0.1])
def test_list_skin_against_fp64(gpu_pkg, orc, skin):
    """Fluid moving at up to 5 m/s, so that with a thin skin the lists are
    rebuilt several times in 100 steps: with any skin, the pairs of a step are
    those within H at the step's positions, and the result holds the FP32
    contract against the FP64 oracle.  Without a skin every step builds."""
    case = gpu_pkg.workloads.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0), layer_ptype=(1, 0, 0))
    spec = _fast_spec(gpu_pkg, case, 5.0)
    ens = gpu_pkg.Ensemble(2, skin=skin)
    assert ens.skin() == skin
    slot = ens.add(spec)
    ens.step(40)
    ens.step(60)
    builds = ens.list_builds(slot)
    if skin == 0.0:
        assert builds == 100
    elif skin == 0.02:
        assert 2 < builds < 60, builds
    else:
        assert 1 <= builds < 20, builds
    ref = _oracle_full(orc, case, 100, spec.v)
    err = errors(ens, slot, ref, case)
    print(f"skin {skin}: {builds} list builds in 100 steps, fp32 vs fp64:", err)
    assert err["rho"] <= TOL and err["v"] <= TOL and err["disp"] <= TOL, err


def test_lists_survive_the_removal_of_an_earlier_instance(gpu_pkg):
    """An instance that keeps its list across a removal in front of it (its
    particles, cell keys and list rows move down) and an admission behind it:
    bit-identical to the same instance alone, same number of list builds."""
    w = gpu_pkg.workloads
    case = w.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0), layer_ptype=(1, 0, 0))
    a = _fast_spec(gpu_pkg, case, 5.0)
    _, b, c, _ = _specs(gpu_pkg)
    alone = gpu_pkg.Ensemble(2, skin=0.02)
    sa = alone.add(a)
    alone.step(27)
    alone.step(23)
    mix = gpu_pkg.Ensemble(2, skin=0.02)
    sb = mix.add(b)
    sm = mix.add(a)
    mix.step(27)
    mix.remove(sb)
    mix.add(c)
    mix.step(23)
    assert mix.list_builds(sm) == alone.list_builds(sa) >= 2
    for f in FIELDS:
        assert np.array_equal(alone.get(sa, f), mix.get(sm, f)), f


def test_skin_is_set_before_instances(gpu_pkg):
    a, _, _, _ = _specs(gpu_pkg)
    ens = gpu_pkg.Ensemble(2)
    assert ens.skin() == pytest.approx(0.05)
    assert gpu_pkg.Ensemble(3).skin() == pytest.approx(0.025)
    ens.add(a)
    with pytest.raises(RuntimeError):
        ens.set_skin(0.2)
