"""Continuous-batching serving loop over the FP32 ensembles.

Requests (dam-break solves with a physical horizon) arrive over time.  Each
is admitted as soon as it has arrived and the device has room for it (free
HBM against the ensemble's bytes per particle), joins the 2-D or 3-D
ensemble, and advances together with every other admitted solve -- one launch
per pass over all of them -- until its horizon; it then leaves, its results
are read back, and its memory admits the next.  Work of requests that arrive
while others run overlaps with theirs on the device.  Reported: time to
horizon per request (arrival to results on the host), p50/p99, and
particle-steps/s over the whole run.

An instance's results do not depend on what else is admitted (the ensemble
keeps instances bit-independent), so a solve gives the same answer alone and
in the mix.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .ensemble import Ensemble, InstanceSpec


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


class ServingLoop:
    """chunk: most steps per ensemble launch sequence between admission
    checks.  reserve: fraction of free HBM left unused.  fields: what to read
    back at the horizon."""

    def __init__(self, chunk: int = 64, reserve: float = 0.1, fields=("x", "v", "rho"), free_bytes=None,
                 ensemble_factory=Ensemble, bytes_per_particle=None):
        self.chunk = int(chunk)
        self.reserve = float(reserve)
        self.fields = tuple(fields)
        self.free_bytes = free_bytes or device_free_bytes
        self.factory = ensemble_factory
        self.bpp = bytes_per_particle or Ensemble.bytes_per_particle
        self.ens = {}
        self.active = {}        # D -> {slot: Request}
        self.remaining = {}     # rid -> steps left

    def _ensemble(self, D):
        if D not in self.ens:
            self.ens[D] = self.factory(D)
            self.active[D] = {}
        return self.ens[D]

    def _fits(self, req: Request) -> bool:
        need = req.spec.n * self.bpp(req.spec.D) * 2  # growth headroom of the buffers
        return need <= (1.0 - self.reserve) * self.free_bytes()

    def run(self, requests, clock=time.perf_counter, idle_sleep=0.0005):
        pending = sorted(requests, key=lambda r: r.arrival)
        t0 = clock()
        steps_done = 0
        while pending or any(self.active.get(D) for D in self.active):
            now = clock() - t0
            # admission: every arrived request that fits, in arrival order
            keep = []
            for req in pending:
                if req.arrival <= now and self._fits(req):
                    ens = self._ensemble(req.spec.D)
                    req.slot = ens.add(req.spec)
                    req.admitted = clock() - t0
                    self.active[req.spec.D][req.slot] = req
                    self.remaining[req.rid] = req.steps
                else:
                    keep.append(req)
            pending = keep
            busy = [D for D in self.active if self.active[D]]
            if not busy:
                if pending and pending[0].arrival <= now:
                    # nothing runs and the device still has no room for it
                    raise RuntimeError(f"request {pending[0].rid} ({pending[0].spec.n} particles) does not fit "
                                       f"in the device's free memory")
                if pending:
                    wait = pending[0].arrival - (clock() - t0)
                    if wait > 0:
                        time.sleep(min(wait, idle_sleep * 20))
                continue
            for D in busy:
                act = self.active[D]
                k = min(self.chunk, min(self.remaining[r.rid] for r in act.values()))
                ens = self.ens[D]
                ens.step(k)
                steps_done += k * sum(r.spec.n for r in act.values())
                for slot, req in list(act.items()):
                    self.remaining[req.rid] -= k
                    if self.remaining[req.rid] == 0:
                        for f in self.fields:
                            req.result[f] = ens.get(slot, f)
                        ens.remove(slot)
                        del act[slot]
                        req.done = clock() - t0
        wall = clock() - t0
        return summarize(requests, wall, steps_done)

    def close(self):
        for e in self.ens.values():
            e.close()
        self.ens.clear()


def summarize(requests, wall: float, particle_steps: int) -> dict:
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
