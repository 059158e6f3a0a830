"""Continuous-batching serving loop over the FP32 ensembles.

Requests (dam-break solves with a horizon in steps) arrive over time.  Each is
admitted as soon as it has arrived and the device has room for it (free HBM
against the ensemble's bytes per particle), joins the 2-D or 3-D ensemble, and
advances together with every other admitted solve -- one launch per pass over
all of them -- until its horizon; it then leaves, its results are read back,
and its memory admits the next.  Work of requests that arrive while others run
overlaps with theirs on the device.  Reported: time to horizon per request
(arrival to results on the host), p50/p99, and particle-steps/s over the run.

The scheduling runs in the library (srv_* in include/gcsph.h: admission,
chunking at the nearest horizon, release).  With the library's ensembles the
whole loop is native; given other ensembles or memory functions (tests on the
host), the same scheduler calls them back through ctypes.

An instance's results do not depend on what else is admitted (the ensemble
keeps instances bit-independent), so a solve gives the same answer alone and
in the mix.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .ensemble import Ensemble, InstanceSpec, _params


@dataclass
class Request:
    rid: int
    arrival: float              # seconds after the loop starts
    spec: InstanceSpec
    steps: int                  # horizon in steps
    admitted: float | None = None
    done: float | None = None
    slot: int | None = None
    result: dict = field(default_factory=dict)

    @property
    def latency(self):
        return None if self.done is None else self.done - self.arrival


def device_free_bytes() -> int:
    import torch
    free, _total = torch.cuda.mem_get_info()
    return int(free)


class _CallbackBackend:
    """The scheduler's backend calling into Python ensembles (host tests)."""

    def __init__(self, loop, requests):
        self.loop = loop
        self.reqs = requests       # native request id -> Request
        self.ens = {}
        self.error = None
        self.table = _lib.gcsph_srv_backend()
        self.table.ctx = None
        self.table.add = _lib.SRV_ADD(self._guard(self._add))
        self.table.remove = _lib.SRV_REMOVE(self._guard(self._remove))
        self.table.step = _lib.SRV_STEP(self._guard(self._step))
        self.table.harvest = _lib.SRV_HARVEST(self._guard(self._harvest))
        self.table.free_bytes = _lib.SRV_FREE(lambda ctx: int(self.loop.free_bytes()))
        self.table.bytes_per_particle = _lib.SRV_BPP(lambda ctx, D: int(self.loop.bpp(D)))

    def _guard(self, fn):
        def call(*a):
            try:
                fn(*a)
                return 0
            except Exception as e:  # noqa: BLE001 -- re-raised by run()
                self.error = e
                return _lib.GCSPH_ESTATE
        return call

    def _ensemble(self, D):
        if D not in self.ens:
            self.ens[D] = self.loop.factory(D)
        return self.ens[D]

    def _add(self, ctx, D, rid, slot):
        req = self.reqs[rid]
        s = self._ensemble(D).add(req.spec)
        req.slot = s
        slot[0] = s

    def _remove(self, ctx, D, slot):
        self.ens[D].remove(slot)

    def _step(self, ctx, D, n):
        self.ens[D].step(n)

    def _harvest(self, ctx, D, slot, rid):
        req = self.reqs[rid]
        for f in self.loop.fields:
            req.result[f] = self.ens[D].get(slot, f)

    def close(self):
        for e in self.ens.values():
            e.close()
        self.ens.clear()


POLICIES = {"arrival": 0, "shortest": 1}


class ServingLoop:
    """chunk: most steps per ensemble launch sequence between admission
    checks.  reserve: fraction of free HBM left unused.  fields: what to read
    back at the horizon.  policy: "arrival" admits in arrival order whatever
    fits; "shortest" admits the smallest work (particles x steps) first while
    a dimension's particles in flight stay within caps = (2-D, 3-D) (0: no
    cap; an idle dimension admits any solve), and a solve that has waited
    max_wait seconds is admitted as soon as it fits, cap or not (0: never).
    free_bytes / ensemble_factory / bytes_per_particle replace the device's
    (host tests)."""

    def __init__(self, chunk: int = 64, reserve: float = 0.1, fields=("x", "v", "rho"), free_bytes=None,
                 ensemble_factory=Ensemble, bytes_per_particle=None, policy: str = "arrival", caps=(0, 0),
                 max_wait: float = 0.0):
        self.chunk = int(chunk)
        self.reserve = float(reserve)
        self.fields = tuple(fields)
        if policy not in POLICIES:
            raise ValueError(f"policy {policy!r} (arrival or shortest)")
        self.policy = policy
        self.caps = (int(caps[0]), int(caps[1]))
        self.max_wait = float(max_wait)
        self.native = free_bytes is None and ensemble_factory is Ensemble and bytes_per_particle is None
        self.free_bytes = free_bytes or device_free_bytes
        self.factory = ensemble_factory
        self.bpp = bytes_per_particle or Ensemble.bytes_per_particle
        self._srv = None
        self._backend = None

    def run(self, requests):
        L = _lib.load()
        reqs = sorted(requests, key=lambda r: r.arrival)
        mask = 0
        for f in self.fields:
            mask |= 1 << _lib.ENS_FIELDS[f]
        self._close_srv()
        h = C.c_void_p()
        if self.native:
            _lib.check(L.srv_create(None, self.chunk, self.reserve, mask, None, C.byref(h)))
        else:
            self._backend = _CallbackBackend(self, {i: r for i, r in enumerate(reqs)})
            _lib.check(L.srv_create(None, self.chunk, self.reserve, mask, C.byref(self._backend.table),
                                    C.byref(h)))
        self._srv = h
        _lib.check(L.srv_set_policy(h, POLICIES[self.policy], self.caps[0], self.caps[1], self.max_wait))
        rid = C.c_int32()
        keep = []  # host arrays referenced until submitted (copied by the library)
        for r in reqs:
            spec = r.spec
            if self.native:
                x = np.ascontiguousarray(spec.x, dtype=np.float64)
                rho = np.ascontiguousarray(spec.rho, dtype=np.float64)
                pt = np.ascontiguousarray(spec.ptype, dtype=np.int32)
                v = None if spec.v is None else np.ascontiguousarray(spec.v, dtype=np.float64)
                p = _params(spec)
                keep.append((x, rho, pt, v))
                _lib.check(L.srv_submit(h, spec.D, spec.n, x.ctypes.data, None if v is None else v.ctypes.data,
                                        rho.ctypes.data, pt.ctypes.data, C.byref(p), int(r.steps),
                                        float(r.arrival), C.byref(rid)))
            else:
                _lib.check(L.srv_submit(h, spec.D, spec.n, None, None, None, None, None, int(r.steps),
                                        float(r.arrival), C.byref(rid)))
        rc = L.srv_run(h)
        if self._backend is not None and self._backend.error is not None:
            raise self._backend.error
        _lib.check(rc)
        st, a, ad, dn = C.c_int32(), C.c_double(), C.c_double(), C.c_double()
        for i, r in enumerate(reqs):
            _lib.check(L.srv_request(h, i, C.byref(st), C.byref(a), C.byref(ad), C.byref(dn)))
            r.admitted = ad.value if ad.value >= 0 else None
            r.done = dn.value if dn.value >= 0 else None
            if self.native and st.value == 2:
                for f in self.fields:
                    comps = r.spec.D if f in ("x", "v") else 1
                    out = np.empty(comps * r.spec.n, dtype=np.float64)
                    _lib.check(L.srv_result(h, i, _lib.ENS_FIELDS[f], out.ctypes.data))
                    r.result[f] = out.reshape(comps, r.spec.n) if comps > 1 else out
        s = _lib.gcsph_srv_stats()
        _lib.check(L.srv_stats(h, C.byref(s)))
        nan = lambda v: None if math.isnan(v) else float(v)  # noqa: E731
        return {
            "requests": int(s.requests),
            "completed": int(s.completed),
            "wall_s": float(s.wall_s),
            "particle_steps": int(s.particle_steps),
            "particle_steps_per_s": s.particle_steps / s.wall_s if s.wall_s > 0 else None,
            "p50_s": nan(s.p50_s),
            "p99_s": nan(s.p99_s),
            "mean_s": nan(s.mean_s),
        }

    def _close_srv(self):
        if self._srv:
            _lib.load().srv_destroy(self._srv)
            self._srv = None
        if self._backend is not None:
            self._backend.close()
            self._backend = None

    def close(self):
        self._close_srv()


def summarize(requests, wall: float, particle_steps: int) -> dict:
    """The loop's statistics from request records (time to horizon: arrival
    to results on the host)."""
    lat = np.array([r.latency for r in requests if r.latency is not None])
    return {
        "requests": len(requests),
        "completed": int(lat.size),
        "wall_s": wall,
        "particle_steps": int(particle_steps),
        "particle_steps_per_s": particle_steps / wall if wall > 0 else None,
        "p50_s": float(np.percentile(lat, 50)) if lat.size else None,
        "p99_s": float(np.percentile(lat, 99)) if lat.size else None,
        "mean_s": float(lat.mean()) if lat.size else None,
    }
