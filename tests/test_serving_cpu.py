"""Host logic of the serving loop (admission, memory gating, exact horizons,
latency bookkeeping) against a fake ensemble -- no GPU."""
import numpy as np


class FakeEnsemble:
    log = []

    def __init__(self, D):
        self.D = D
        self.slots = {}
        self.next = 0

    def add(self, spec):
        s = self.next
        self.next += 1
        self.slots[s] = [spec, 0]
        FakeEnsemble.log.append(("add", self.D, spec.n))
        return s

    def remove(self, slot):
        FakeEnsemble.log.append(("remove", self.D, self.slots[slot][0].n, self.slots[slot][1]))
        del self.slots[slot]

    def step(self, k):
        for v in self.slots.values():
            v[1] += k

    def get(self, slot, f):
        return np.full(3, float(self.slots[slot][1]))

    def close(self):
        pass


class Spec:
    def __init__(self, D, n):
        self.D, self.n = D, n


def _loop(pkg, **kw):
    FakeEnsemble.log = []
    return pkg.serving.ServingLoop(ensemble_factory=FakeEnsemble, bytes_per_particle=lambda D: 100, **kw)


def test_every_request_reaches_exactly_its_horizon(pkg):
    S = pkg.serving
    reqs = [S.Request(i, 0.0, Spec(2 if i % 3 else 3, 1000 + i), steps) for i, steps in
            enumerate([5, 130, 64, 1, 77, 200])]
    loop = _loop(pkg, chunk=64, free_bytes=lambda: 10 ** 12)
    stats = loop.run(reqs)
    assert stats["completed"] == len(reqs)
    removed = {(n, steps) for (tag, D, n, *rest) in FakeEnsemble.log if tag == "remove" for steps in rest}
    assert removed == {(r.spec.n, r.steps) for r in reqs}
    for r in reqs:
        assert r.result["x"][0] == r.steps
        assert r.latency is not None and r.latency >= 0
    assert stats["particle_steps"] == sum(r.spec.n * r.steps for r in reqs)
    assert stats["p50_s"] is not None and stats["p99_s"] >= stats["p50_s"]


def test_admission_waits_for_memory(pkg):
    """Only one request fits at a time: the second is admitted only after the
    first has left, never alongside it."""
    S = pkg.serving
    reqs = [S.Request(0, 0.0, Spec(2, 1000), 10), S.Request(1, 0.0, Spec(2, 1000), 10)]
    def live():
        return (sum(1 for t in FakeEnsemble.log if t[0] == "add")
                - sum(1 for t in FakeEnsemble.log if t[0] == "remove"))

    # 1000 particles x 100 B x 2 = 2e5 B per request; 3e5 B free when idle
    loop = _loop(pkg, chunk=4, free_bytes=lambda: 3 * 10 ** 5 - live() * 2 * 10 ** 5, reserve=0.0)
    loop.run(reqs)
    tags = [t[0] for t in FakeEnsemble.log]
    assert tags == ["add", "remove", "add", "remove"], tags


def test_arrivals_in_the_future_are_waited_for(pkg):
    S = pkg.serving
    reqs = [S.Request(0, 0.05, Spec(2, 10), 3)]
    loop = _loop(pkg, free_bytes=lambda: 10 ** 12)
    stats = loop.run(reqs)
    assert reqs[0].admitted >= 0.05
    assert stats["completed"] == 1


def test_a_request_that_can_never_fit_is_refused(pkg):
    import pytest
    S = pkg.serving
    reqs = [S.Request(0, 0.0, Spec(2, 10 ** 6), 3)]
    loop = _loop(pkg, free_bytes=lambda: 10 ** 6)
    with pytest.raises(RuntimeError):
        loop.run(reqs)


def _live(D=None):
    """Particles in flight per the fake ensemble's log (of one dimension, or all)."""
    n = 0
    for t in FakeEnsemble.log:
        if D is not None and t[1] != D:
            continue
        n += t[2] if t[0] == "add" else -t[2]
    return n


def test_shortest_first_admits_small_work_first_within_the_cap(pkg):
    """All requests arrive at once.  Under the shortest-first policy the
    smallest work (particles x steps) is admitted first, the 2-D particles in
    flight never pass the cap while another solve runs, and a solve larger
    than the cap runs alone once its dimension is idle."""
    S = pkg.serving
    sizes = [(4000, 10), (500, 20), (1500, 5), (9000, 3), (800, 40), (3000, 2)]  # (n, steps), all 2-D
    reqs = [S.Request(i, 0.0, Spec(2, n), steps) for i, (n, steps) in enumerate(sizes)]
    cap = 5000
    peaks = []
    orig_step = FakeEnsemble.step

    def step(self, k):
        peaks.append(_live(2))
        orig_step(self, k)

    FakeEnsemble.step = step
    try:
        loop = _loop(pkg, chunk=64, free_bytes=lambda: 10 ** 12, policy="shortest", caps=(cap, 0))
        stats = loop.run(reqs)
    finally:
        FakeEnsemble.step = orig_step
    assert stats["completed"] == len(reqs)
    adds = [t[2] for t in FakeEnsemble.log if t[0] == "add"]
    # the first admission is the smallest work, 3000 particles x 2 steps
    works = sorted((n * st, n) for n, st in sizes)
    assert adds[0] == works[0][1]
    for p in peaks:
        assert p <= cap or p == 9000, peaks  # the 9000-particle solve only alone
    assert 9000 in peaks
    for r in reqs:
        assert r.result["x"][0] == r.steps


def test_arrival_policy_admits_everything_that_fits(pkg):
    S = pkg.serving
    reqs = [S.Request(i, 0.0, Spec(2, 1000 * (i + 1)), 10 - i) for i in range(4)]
    loop = _loop(pkg, chunk=64, free_bytes=lambda: 10 ** 12)
    loop.run(reqs)
    tags = [t[0] for t in FakeEnsemble.log]
    assert tags[:4] == ["add"] * 4
    assert [t[2] for t in FakeEnsemble.log[:4]] == [1000, 2000, 3000, 4000]


def test_policy_round_trip_and_bad_policy(pkg):
    import ctypes as C
    import pytest
    L = pkg._lib.load()
    h = C.c_void_p()
    tbl = pkg.serving._CallbackBackend(_loop(pkg), {}).table
    pkg._lib.check(L.srv_create(None, 8, 0.1, 0, C.byref(tbl), C.byref(h)))
    try:
        pkg._lib.check(L.srv_set_policy(h, 1, 123, 456, 2.5))
        p, a, b, w = C.c_int32(), C.c_int64(), C.c_int64(), C.c_double()
        pkg._lib.check(L.srv_get_policy(h, C.byref(p), C.byref(a), C.byref(b), C.byref(w)))
        assert (p.value, a.value, b.value, w.value) == (1, 123, 456, 2.5)
        assert L.srv_set_policy(h, 7, 0, 0, 0.0) != 0
        assert L.srv_set_policy(h, 1, -1, 0, 0.0) != 0
        assert L.srv_set_policy(h, 1, 0, 0, -1.0) != 0
    finally:
        L.srv_destroy(h)
    with pytest.raises(ValueError):
        pkg.serving.ServingLoop(policy="fastest")


def test_shortest_first_max_wait_lifts_the_cap(pkg):
    """A solve that has waited max_wait is admitted though the cap is full:
    with a wait limit already passed at the first round, every solve is
    admitted at once, as under arrival order."""
    S = pkg.serving
    reqs = [S.Request(i, 0.0, Spec(2, 1000 * (i + 1)), 10) for i in range(4)]
    loop = _loop(pkg, chunk=64, free_bytes=lambda: 10 ** 12, policy="shortest", caps=(1000, 0), max_wait=1e-9)
    loop.run(reqs)
    assert [t[0] for t in FakeEnsemble.log[:4]] == ["add"] * 4
    # without the wait limit the 1000-particle cap admits one solve at a time
    reqs = [S.Request(i, 0.0, Spec(2, 1000 * (i + 1)), 10) for i in range(4)]
    loop = _loop(pkg, chunk=64, free_bytes=lambda: 10 ** 12, policy="shortest", caps=(1000, 0))
    loop.run(reqs)
    assert [t[0] for t in FakeEnsemble.log] == ["add", "remove"] * 4


def test_latency_statistics_match_numpy(pkg):
    """p50/p99/mean time to horizon from the native scheduler equal numpy's
    (linear percentile) over the requests' own arrival-to-done times."""
    S = pkg.serving
    reqs = [S.Request(i, 0.002 * i, Spec(2 if i % 2 else 3, 100 + 37 * i), 3 + (7 * i) % 20) for i in range(13)]
    loop = _loop(pkg, chunk=4, free_bytes=lambda: 10 ** 12, policy="shortest", caps=(600, 400))
    stats = loop.run(reqs)
    lat = np.array([r.done - r.arrival for r in reqs])
    assert stats["completed"] == len(reqs)
    assert abs(stats["p50_s"] - np.percentile(lat, 50)) <= 1e-12
    assert abs(stats["p99_s"] - np.percentile(lat, 99)) <= 1e-12
    assert abs(stats["mean_s"] - lat.mean()) <= 1e-12
