"""Long-horizon checks on the 2-D dam break (dx = 0.02, 6,518 particles,
cell list rebuilt every step): 1,000 steps as one stepsolve!(prob, 1000)
call, the configuration's full horizon.  Point-wise parity stops meaning
much as the flow develops, so the checks are the fluid's total mass inside
the tank, its kinetic energy, the change of its mechanical energy and the
surge front (diagnostics.py), each with the tolerance stated there:
  * the FP64 drop-in against the oracle over the same 1,000 steps;
  * the batched FP32 path against the FP64 drop-in over the same steps.
The reference loop that produces such horizons is timesolve!,
src/sphproblem.jl:420-511 (stepsolve! batches, src/sphproblem.jl:204-345)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

STEPS = 1000


def _gpu_summary(pkg, prob, case):
    D = pkg.diagnostics
    x = torch.stack(prob.system.points).cpu().numpy()
    v = torch.stack(prob.v).cpu().numpy()
    return D.flow_summary(x, v, prob.rho.cpu().numpy(), case.ptype, case.m0, case.g, case.interior)


@pytest.fixture(scope="module")
def c1_runs(gpu_pkg, orc):
    """The FP64 drop-in (default split rows) and the oracle, 1,000 steps each."""
    g = gpu_pkg
    case = g.workloads.dam_break_2d()
    start = g.diagnostics.flow_summary(case.x, np.zeros_like(case.x), case.rho, case.ptype, case.m0, case.g,
                                       case.interior)
    system = g.GPUCellList(tuple(case.x), case.cellsize, case.dist)
    prob = g.SPHProblem(system, case.dx, case.h, case.H, g.WendlandC2(dim=2), case.rho, case.ptype, case.rho0,
                        case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL)
    un, _ = prob.stepsolve(STEPS)
    assert un == STEPS
    fp64 = _gpu_summary(g, prob, case)
    p = orc.default_params(case.dx, case.h, case.H, case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma,
                           case.delta, case.CFL, case.dist)
    ref = orc.OracleSystem(case.x, case.cellsize, case.dist, case.rho, case.ptype, p)
    ref.stepsolve(STEPS)
    oracle = g.diagnostics.flow_summary(ref.get("x"), ref.get("v"), ref.get("rho"), case.ptype, case.m0, case.g,
                                        case.interior)
    prob.close()
    system.close()
    return case, start, fp64, oracle


def test_fp64_long_horizon_matches_oracle(gpu_pkg, c1_runs):
    case, start, fp64, oracle = c1_runs
    D = gpu_pkg.diagnostics
    diff = D.compare_summaries(fp64, oracle, start)
    print(f"\nFP64 vs oracle after {STEPS} steps: {diff}\n  fp64 {fp64}\n  oracle {oracle}")
    assert fp64["fluid_in_tank"] == oracle["fluid_in_tank"] == start["fluid_in_tank"]
    # the flow has developed: with ptype-0 walls the boundary force (r0 = 2dx,
    # more than the gap to the first fluid row) throws the bottom rows up at
    # the start, so the potential energy moves away from its initial value
    assert oracle["kinetic"] > 0 and abs(oracle["potential"] - start["potential"]) > 1.0
    bad = D.within(diff, D.TOL_FP64)
    assert not bad, f"over tolerance: {bad}"


def test_fp32_ensemble_long_horizon_matches_fp64(gpu_pkg, c1_runs):
    case, start, fp64, _ = c1_runs
    g = gpu_pkg
    D = g.diagnostics
    ens = g.Ensemble(2)
    slot = ens.add(g.spec_from_case(case))
    ens.step(STEPS)
    fp32 = D.flow_summary(ens.get(slot, "x"), ens.get(slot, "v"), ens.get(slot, "rho"), case.ptype, case.m0, case.g,
                          case.interior)
    ens.close()
    diff = D.compare_summaries(fp32, fp64, start)
    print(f"\nFP32 ensemble vs FP64 after {STEPS} steps: {diff}\n  fp32 {fp32}")
    assert fp32["fluid_in_tank"] == fp64["fluid_in_tank"]
    bad = D.within(diff, D.TOL_FP32)
    assert not bad, f"over tolerance: {bad}"
