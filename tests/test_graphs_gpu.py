"""Captured stepsolve! calls (one CUDA graph per call) against the per-step
host loop and against the oracle.

Where update! follows every step (nui = dist - H = 0), sph_step runs the whole
call as one graph and moves the loop's host decisions to the device.  The
arithmetic is the same kernels in the same order, so every field, updaten and
max|cΔx| must be bit-identical to the per-step loop, call after call (cache
hits, and the re-sorts' buffer parity alternating between calls).
"""
import numpy as np
import pytest
import torch

from test_sph_gpu import FIELDS, check, gpu_field, make_pair, run_both

pytestmark = pytest.mark.gpu


def _twins(pkg, case, lanes):
    out = []
    for graphs in (True, False):
        system = pkg.GPUCellList(tuple(case.x), case.cellsize, case.dist)
        prob = pkg.SPHProblem(system, case.dx, case.h, case.H, pkg.WendlandC2(dim=case.D), case.rho, case.ptype,
                              case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL,
                              g=case.g, s=case.s)
        prob.set_lanes(lanes)
        prob.set_graphs(graphs)
        for k, val in case.extra.items():
            setattr(prob, k, val)
        out.append(prob)
    return out


@pytest.mark.parametrize("lanes", [1, 0])
@pytest.mark.parametrize("timestepping", [False, True])
def test_graph_calls_match_host_loop(gpu_pkg, lanes, timestepping):
    case = gpu_pkg.workloads.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0), layer_ptype=(1, 0, 0))
    assert case.dist - case.H == 0.0
    g, e = _twins(gpu_pkg, case, lanes)
    for n in (7, 7, 4, 7, 1):
        a = g.stepsolve(n, timestepping=timestepping)
        b = e.stepsolve(n, timestepping=timestepping)
        assert a == b, (n, a, b)
        assert g.etime == e.etime and g.dt == e.dt
        for name in FIELDS:
            x, y = gpu_field(g, name), gpu_field(e, name)
            assert np.array_equal(x, y), (n, name, np.abs(x - y).max())
        assert g.system.pairsn == e.system.pairsn
    caps, reps = g.graph_stats()
    assert reps >= 4 and 1 <= caps <= reps, (caps, reps)  # the first call runs per step (buffers unsized)
    assert e.graph_stats() == (0, 0)


def test_graph_matches_oracle_exact(gpu_pkg, orc):
    """lanes = 1 through graphs stays bit-identical to the oracle over several
    calls (100 steps)."""
    case = gpu_pkg.workloads.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0), layer_ptype=(1, 0, 0))
    prob, ref = make_pair(gpu_pkg, orc, case, lanes=1)
    prob.set_graphs(True)
    for n in (1, 33, 33, 33):
        run_both(prob, ref, n)
    check(orc, prob, ref, case, 1, [(100, {})])
    assert prob.graph_stats()[1] == 3


@pytest.mark.parametrize("lanes", [1, 4])
def test_graph_overflow_falls_back(gpu_pkg, orc, lanes):
    """A call whose first update! outgrows the neighbour buffers inside the
    graph: every later kernel skips, the caller's arrays keep the call's
    inputs, the library grows the buffers and runs the call again per step.
    The particles are spread out for one step (small buffers), then put back
    close together.  Against the same sequence without graphs (bit-identical)
    and, for lanes = 1, the oracle doing the same (bit-identical)."""
    case = gpu_pkg.workloads.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0), layer_ptype=(1, 0, 0))
    centre = case.x.mean(axis=1, keepdims=True)
    spread = np.ascontiguousarray(centre + 3.0 * (case.x - centre))
    probs = []
    for graphs in (True, False):
        system = gpu_pkg.GPUCellList(tuple(spread), case.cellsize, case.dist)
        prob = gpu_pkg.SPHProblem(system, case.dx, case.h, case.H, gpu_pkg.WendlandC2(dim=2), case.rho, case.ptype,
                                  case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL)
        prob.set_lanes(lanes)
        prob.set_graphs(graphs)
        probs.append(prob)
    p = orc.default_params(case.dx, case.h, case.H, case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma,
                           case.delta, case.CFL, case.dist)
    ref = orc.OracleSystem(spread, case.cellsize, case.dist, case.rho, case.ptype, p)
    g, e = probs

    def both(n):
        a, b = g.stepsolve(n), e.stepsolve(n)
        assert a == b, (n, a, b)
        if lanes == 1:
            run_ref = ref.stepsolve(n)
            assert run_ref[0] == a[0] and run_ref[1] == a[1], (a, run_ref)

    both(1)
    few = g.system.pairsn
    for prob in probs:
        for d in range(case.D):
            prob.system.points[d].copy_(torch.from_numpy(np.ascontiguousarray(case.x[d])))
    ref.set_x(case.x)
    both(10)
    assert g.graph_stats() == (1, 0)  # captured, replay overflowed, call ran per step
    assert g.system.pairsn > 2 * few
    both(5)  # grown buffers: a graph again
    assert g.graph_stats() == (2, 1)
    for name in FIELDS:
        x, y = gpu_field(g, name), gpu_field(e, name)
        assert np.array_equal(x, y), (name, np.abs(x - y).max())
    if lanes == 1:
        check(orc, g, ref, case, 1, [])
