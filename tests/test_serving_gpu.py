"""The serving loop on the device: requests that arrive while others run are
admitted into the running ensembles, each reaches its horizon, and each
result is the same alone and in the mix (bit-identical: the ensemble keeps
instances independent), 2-D and 3-D requests side by side."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(pkg):
    S, w = pkg.serving, pkg.workloads
    # the first three arrive together (admitted side by side), the rest while they run or after
    cases = [
        (0.00, w.sized_dam_break_2d(3000, 2.0, 0.02), 60),
        (0.00, w.sized_dam_break_3d(2000, 1.0, 0.03), 45),
        (0.00, w.sized_dam_break_2d(8000, 0.7, 0.01), 80),
        (0.05, w.sized_dam_break_2d(2500, 3.0, 0.015), 33),
        (0.06, w.sized_dam_break_3d(3000, 2.0, 0.02), 70),
    ]
    return [S.Request(i, t, pkg.spec_from_case(c), n) for i, (t, c, n) in enumerate(cases)]


def test_requests_in_the_mix_match_each_run_alone(gpu_pkg):
    S = gpu_pkg.serving
    reqs = _requests(gpu_pkg)
    loop = S.ServingLoop(chunk=16)
    stats = loop.run(reqs)
    loop.close()
    assert stats["completed"] == len(reqs)
    assert stats["p99_s"] >= stats["p50_s"] > 0
    assert stats["particle_steps"] == sum(r.spec.n * r.steps for r in reqs)
    # overlap: requests that arrived together ran side by side
    assert max(r.admitted for r in reqs[:3]) < min(r.done for r in reqs[:3])
    for r in reqs:
        ens = gpu_pkg.Ensemble(r.spec.D)
        s = ens.add(r.spec)
        ens.step(r.steps)
        for f in ("x", "v", "rho"):
            assert np.array_equal(ens.get(s, f), r.result[f]), (r.rid, f)
        ens.close()
