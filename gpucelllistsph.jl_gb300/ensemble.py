"""Batched FP32 ensemble: many independent SPH instances stepped together.

The reference advances one SPHProblem per stepsolve! call
(src/sphproblem.jl:204-345); an Ensemble keeps every admitted instance
resident on the device and advances all of them with one launch per pass
(include/gcsph.h, ens_*).  Pair arithmetic in FP32 with Kahan-compensated
sums, density held as ρ - ρ₀, positions in FP64.  Instances come and go
(admission, retirement) without disturbing the others: an instance's results
are bit-identical whether it runs alone or in a mix.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib


@dataclass
class InstanceSpec:
    """One dam-break-style solve: particles, parameters and its frozen grid."""
    x: np.ndarray            # (D, n) float64
    rho: np.ndarray          # (n,)
    ptype: np.ndarray        # (n,) int32
    dx: float
    h: float
    H: float
    rho0: float
    m0: float
    dt: float
    alpha: float
    c0: float
    gamma: int = 7
    delta: float = 0.1
    g: float = 9.81
    nu: float = 0.0
    s: float = 0.0
    bound_D: float = 0.4
    bound_l: float = 0.0     # 0: 2 dx
    cspmn: int = 15          # cspmcorr! period in steps (SPHProblem's default), 0 = never
    dpc_l0: float = 0.0      # dpcreg! when > 0 (SPHProblem's defaults below)
    dpc_pmin: float = 1.0
    dpc_pmax: float = 10000.0
    dpc_lambda: float = 0.01
    xsph_eps: float = 0.0    # xsphcorr! when > 0
    v: np.ndarray | None = None
    grid_min: tuple | None = None
    grid_max: tuple | None = None

    @property
    def D(self):
        return self.x.shape[0]

    @property
    def n(self):
        return self.x.shape[1]


def spec_from_case(case, dt=None, alpha=None, delta=None, margin_cells=2, headroom=0.5):
    """An InstanceSpec from a workloads.Case.  The frozen grid is the particle
    bounding box plus `margin_cells` cells on every side and `headroom` times
    the box height above (splashes clamp into the top row beyond it)."""
    D = case.x.shape[0]
    lo = case.x.min(axis=1) - margin_cells * case.H
    hi = case.x.max(axis=1) + margin_cells * case.H
    hi[1] += headroom * (hi[1] - lo[1])
    ex = dict(case.extra) if getattr(case, "extra", None) else {}
    extra = {k: float(ex[k]) for k in ("dpc_l0", "dpc_pmin", "dpc_pmax", "dpc_lambda", "xsph_eps") if k in ex}
    if "cspmn" in ex:
        extra["cspmn"] = int(ex["cspmn"])
    return InstanceSpec(x=case.x, rho=case.rho, ptype=case.ptype, dx=case.dx, h=case.h, H=case.H, rho0=case.rho0,
                        m0=case.m0, dt=case.dt if dt is None else dt, alpha=case.alpha if alpha is None else alpha,
                        c0=case.c0, gamma=case.gamma, delta=case.delta if delta is None else delta, g=case.g,
                        nu=ex.get("nu", 0.0), s=getattr(case, "s", 0.0) or 0.0,
                        grid_min=tuple(lo[:D]), grid_max=tuple(hi[:D]), **extra)


def _params(spec: InstanceSpec) -> _lib.gcsph_ens_params:
    p = _lib.gcsph_ens_params()
    for k in ("dx", "h", "H", "rho0", "m0", "dt", "alpha", "nu", "g", "c0", "s", "delta", "bound_D"):
        setattr(p, k, float(getattr(spec, k)))
    p.bound_l = float(spec.bound_l) if spec.bound_l > 0 else 2.0 * float(spec.dx)
    p.gamma = int(spec.gamma)
    p.cspmn = int(spec.cspmn)
    for k in ("dpc_l0", "dpc_pmin", "dpc_pmax", "dpc_lambda", "xsph_eps"):
        setattr(p, k, float(getattr(spec, k)))
    lo = spec.grid_min if spec.grid_min is not None else spec.x.min(axis=1) - 2 * spec.H
    hi = spec.grid_max if spec.grid_max is not None else spec.x.max(axis=1) + 2 * spec.H
    for d in range(spec.D):
        p.grid_min[d] = float(lo[d])
        p.grid_max[d] = float(hi[d])
    return p


class Ensemble:
    def __init__(self, D: int, stream: int = 0, skin: float | None = None):
        self.D = int(D)
        h = C.c_void_p()
        _lib.check(_lib.load().ens_create(self.D, C.c_void_p(stream), C.byref(h)))
        self._h = h
        self.specs = {}
        if skin is not None:
            self.set_skin(skin)

    @staticmethod
    def bytes_per_particle(D: int) -> int:
        b = C.c_int64()
        _lib.check(_lib.load().ens_bytes_per_particle(int(D), C.byref(b)))
        return int(b.value)

    def add(self, spec: InstanceSpec) -> int:
        if spec.D != self.D:
            raise ValueError("instance dimension differs from the ensemble's")
        x = np.ascontiguousarray(spec.x, dtype=np.float64)
        rho = np.ascontiguousarray(spec.rho, dtype=np.float64)
        pt = np.ascontiguousarray(spec.ptype, dtype=np.int32)
        v = None if spec.v is None else np.ascontiguousarray(spec.v, dtype=np.float64)
        slot = C.c_int32()
        p = _params(spec)
        _lib.check(_lib.load().ens_add(self._h, x.shape[1], x.ctypes.data, None if v is None else v.ctypes.data,
                                       rho.ctypes.data, pt.ctypes.data, C.byref(p), C.byref(slot)))
        self.specs[slot.value] = spec
        return int(slot.value)

    def remove(self, slot: int):
        _lib.check(_lib.load().ens_remove(self._h, int(slot)))
        self.specs.pop(int(slot), None)

    def step(self, n: int = 1):
        _lib.check(_lib.load().ens_step(self._h, int(n)))

    def get(self, slot: int, field: str) -> np.ndarray:
        spec = self.specs[int(slot)]
        comps = self.D if field in ("x", "v") else 1
        out = np.empty(comps * spec.n, dtype=np.float64)
        _lib.check(_lib.load().ens_get(self._h, int(slot), _lib.ENS_FIELDS[field], out.ctypes.data))
        return out.reshape(comps, spec.n) if comps > 1 else out

    def info(self, slot: int):
        n, steps, t = C.c_int64(), C.c_int64(), C.c_double()
        _lib.check(_lib.load().ens_info(self._h, int(slot), C.byref(n), C.byref(steps), C.byref(t)))
        return {"n": int(n.value), "steps": int(steps.value), "etime": float(t.value)}

    def totals(self):
        a, b, c = C.c_int32(), C.c_int64(), C.c_int64()
        _lib.check(_lib.load().ens_totals(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return {"instances": int(a.value), "particles": int(b.value), "cells": int(c.value)}

    def set_tuning(self, tpb: int = 0, graphs: bool = True):
        _lib.check(_lib.load().ens_set_tuning(self._h, int(tpb), int(bool(graphs))))

    def tuning(self):
        t, L, a, b = C.c_int32(), C.c_int32(), C.c_int64(), C.c_int64()
        lib = _lib.load()
        _lib.check(lib.ens_get_tuning(self._h, C.byref(t), C.byref(L), C.byref(a), C.byref(b)))
        c, d, k = C.c_int32(), C.c_int32(), C.c_int32()
        _lib.check(lib.ens_get_list_build(self._h, None, C.byref(c), C.byref(d), C.byref(k)))
        return {"tpb": int(t.value), "list_lanes": int(L.value), "cells_per_block": int(c.value),
                "staging_depth": int(d.value), "tile_capacity": int(k.value), "captures": int(a.value),
                "replays": int(b.value)}

    def set_list_build(self, lanes: int = 0, cells_per_block: int = 0, depth: int = 1, capacity: int = 0):
        """Fix the neighbour-list build (lanes = 0: autotuned).  cells_per_block
        0 = a thread group per particle; 2/4/8/16 = a block per tile of that
        many cells, the neighbourhood staged in shared memory, `depth` tiles at
        a time; `capacity` = particles a tile buffer holds (0: from (H/dx)^D).
        Results do not depend on the choice."""
        _lib.check(_lib.load().ens_set_list_build(self._h, int(lanes), int(cells_per_block), int(depth),
                                                  int(capacity)))

    def set_skin(self, skin: float):
        """List skin: cells and neighbour lists of radius H (1 + skin), rebuilt
        per instance once a particle has moved about skin H / 2 (0: every
        step).  Set before the first add."""
        _lib.check(_lib.load().ens_set_skin(self._h, float(skin)))

    def skin(self) -> float:
        v = C.c_double()
        _lib.check(_lib.load().ens_get_skin(self._h, C.byref(v)))
        return float(v.value)

    def list_builds(self, slot: int) -> int:
        """How many times the instance's cells and list were built."""
        v = C.c_int64()
        _lib.check(_lib.load().ens_list_builds(self._h, int(slot), C.byref(v)))
        return int(v.value)

    def set_dpc_bound(self, on: bool):
        """dpcreg!'s row bound: skip the rows that can hold no pair within l0
        after the step (on by default).  Results are the same either way."""
        _lib.check(_lib.load().ens_set_dpc_bound(self._h, 1 if on else 0))

    def dpc_bound(self) -> bool:
        v = C.c_int32()
        _lib.check(_lib.load().ens_get_dpc_bound(self._h, C.byref(v)))
        return bool(v.value)

    def set_list_stride(self, nls: int):
        _lib.check(_lib.load().ens_set_list_stride(self._h, int(nls)))

    def list_stride(self) -> int:
        n = C.c_int32()
        _lib.check(_lib.load().ens_get_list_stride(self._h, C.byref(n)))
        return int(n.value)

    def close(self):
        h = self.__dict__.get("_h")
        if h:
            _lib.load().ens_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass
