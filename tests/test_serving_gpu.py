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


def test_incremental_serving_through_the_c_abi(gpu_pkg):
    """A server's use of the scheduler: submit as requests arrive, call
    srv_progress in its own loop, read each result when it is done -- through
    the C ABI; every result equals the same solve alone."""
    import ctypes as C
    L = gpu_pkg._lib.load()
    lib = gpu_pkg._lib
    w = gpu_pkg.workloads
    cases = [(w.sized_dam_break_2d(3000, 2.0, 0.02), 40), (w.sized_dam_break_3d(2000, 1.0, 0.03), 30),
             (w.sized_dam_break_2d(2500, 3.0, 0.015), 25)]
    specs = [gpu_pkg.spec_from_case(c) for c, _ in cases]
    h = C.c_void_p()
    lib.check(L.srv_create(None, 8, 0.1, 0x7, None, C.byref(h)))
    keep, rids = [], []

    def submit(k):
        s, n = specs[k], cases[k][1]
        x = np.ascontiguousarray(s.x, dtype=np.float64)
        rho = np.ascontiguousarray(s.rho, dtype=np.float64)
        pt = np.ascontiguousarray(s.ptype, dtype=np.int32)
        p = gpu_pkg.ensemble._params(s)
        keep.append((x, rho, pt, p))
        rid = C.c_int32()
        lib.check(L.srv_submit(h, s.D, s.n, x.ctypes.data, None, rho.ctypes.data, pt.ctypes.data, C.byref(p), n,
                               -1.0, C.byref(rid)))
        rids.append(rid.value)

    running, queued = C.c_int32(), C.c_int32()
    submit(0)
    submit(1)
    lib.check(L.srv_progress(h, C.byref(running), C.byref(queued)))
    assert running.value == 2 and queued.value == 0
    submit(2)                                   # arrives while the others run
    rounds = 0
    while True:
        lib.check(L.srv_progress(h, C.byref(running), C.byref(queued)))
        rounds += 1
        if running.value == 0 and queued.value == 0:
            break
        assert rounds < 1000
    state = C.c_int32()
    for k, rid in enumerate(rids):
        lib.check(L.srv_request(h, rid, C.byref(state), None, None, None))
        assert state.value == 2
        s, n = specs[k], cases[k][1]
        ens = gpu_pkg.Ensemble(s.D)
        slot = ens.add(s)
        ens.step(n)
        for f, code in (("x", 0), ("v", 1), ("rho", 2)):
            comps = s.D if f in ("x", "v") else 1
            out = np.empty(comps * s.n)
            lib.check(L.srv_result(h, rid, code, out.ctypes.data))
            assert np.array_equal(out.reshape(comps, s.n) if comps > 1 else out, ens.get(slot, f)), (k, f)
        ens.close()
    st = lib.gcsph_srv_stats()
    lib.check(L.srv_stats(h, C.byref(st)))
    assert st.completed == 3 and st.particle_steps == sum(s.n * n for s, (_, n) in zip(specs, cases))
    L.srv_destroy(h)
