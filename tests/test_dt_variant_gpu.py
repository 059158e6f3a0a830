"""Δt_stepping's optional pair-relative velocity bound: after a timestepping
call, Δt equals CFL·min(√(h/3 max|a|), h/(c₀ + max over pairs
|h Δv·Δx/(|Δx|²+η²)|)) clamped to the limits, recomputed here from the
final state and the step's pair list; the default stays the reference's
formula (absolute v·x)."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _problem(pkg, case, v):
    system = pkg.GPUCellList(tuple(case.x), case.cellsize, case.dist)
    prob = pkg.SPHProblem(system, case.dx, case.h, case.H, pkg.WendlandC2(dim=2), case.rho, case.ptype, case.rho0,
                          case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL, v=tuple(v))
    return system, prob


@pytest.mark.parametrize("relative", [False, True])
def test_dt_from_final_state(gpu_pkg, relative):
    case = gpu_pkg.workloads.dam_break_2d(dx=0.04, fluid=(0.6, 0.8), tank=(1.2, 1.0))
    rng = np.random.default_rng(4)
    v = rng.uniform(-0.3, 0.3, case.x.shape)
    v[:, case.ptype <= 1] = 0.0
    system, prob = _problem(gpu_pkg, case, v)
    prob.set_dt_variant(relative)
    lims = (1e-9, prob.CFL * prob.H / (3 * prob.c0))
    prob.stepsolve(6, timestepping=True, timelims=lims)
    x = torch.stack(system.points).cpu().numpy()
    vv = torch.stack(prob.v).cpu().numpy()
    a = torch.stack(prob.field("a")).cpu().numpy()
    h, eta2 = prob.h, (0.01 * prob.h) ** 2
    amax = np.sqrt((a * a).sum(axis=0)).max()
    if relative:
        pr = gpu_pkg.neighborlistview(system).cpu().numpy().astype(np.int64) - 1
        i, j = pr[:, 0], pr[:, 1]
        dx, dv = x[:, i] - x[:, j], vv[:, i] - vv[:, j]
        vmax = np.abs(h * (dv * dx).sum(axis=0) / ((dx * dx).sum(axis=0) + eta2)).max()
    else:
        vmax = np.abs(h * (vv * x).sum(axis=0) / ((x * x).sum(axis=0) + eta2)).max()
    want = prob.CFL * min(math.sqrt(h / (3 * amax)), h / (prob.c0 + vmax))
    want = min(max(want, lims[0]), lims[1])
    assert abs(prob.dt - want) <= 1e-12 * want, (prob.dt, want)
