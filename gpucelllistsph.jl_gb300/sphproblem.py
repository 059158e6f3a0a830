"""SPHProblem, stepsolve!, timesolve! -- host-side mirror of src/sphproblem.jl.

The mutable scalar fields map onto the library's gcsph_params; the array
fields are the caller's CUDA tensors (ρ, v, ptype, and the cell list's points)
plus library-owned work arrays read through the getters.  Python names:
ρ -> rho, Δt -> dt, 𝜈 -> nu, δᵩ -> delta, γ -> gamma, xsph_𝜀 -> xsph_eps,
dpc_l₀ -> dpc_l0, dpc_λ -> dpc_lambda, stepsolve! -> stepsolve.
"""
from __future__ import annotations

import ctypes as C
import math
import time
import warnings

import torch

from . import _lib
from .celllist import GPUCellList

_EPS = 2.220446049250313e-16


class WendlandC2:
    """Kernel descriptor standing in for SPHKernels.jl's WendlandC2(T, dim)."""

    def __init__(self, T=torch.float64, dim: int = 2):
        if dim not in (2, 3):
            raise ValueError("WendlandC2 is defined here for dim 2 and 3")
        self.T = T
        self.dim = int(dim)

    def __repr__(self):
        return f"WendlandC2(Float64, {self.dim})"


def _cuda_f64(t, n, name):
    t = torch.as_tensor(t)
    if t.numel() != n:
        raise ValueError(f"length({name}) ({t.numel()}) != N ({n})")
    if t.device.type != "cuda" or t.dtype != torch.float64 or not t.is_contiguous():
        t = t.to(device="cuda", dtype=torch.float64).contiguous()
    return t


_PARAM_FIELDS = ("dx", "h", "H", "rho0", "m0", "dt", "alpha", "nu", "g", "c0", "s", "delta", "CFL", "nui", "etime",
                 "dpc_l0", "dpc_pmin", "dpc_pmax", "dpc_lambda", "xsph_eps", "bound_D", "bound_l", "gamma", "cspmn")


class SPHProblem:
    """SPHProblem(system, dx, h, H, sphkernel, ρ, ptype, ρ₀, m₀, Δt, α, c₀, γ, δᵩ, CFL; v, g, s)
    -- src/sphproblem.jl:113-192 (defaults :172-191)."""

    def __init__(self, system: GPUCellList, dx, h, H, sphkernel, rho, ptype, rho0, m0, dt, alpha, c0, gamma,
                 delta, CFL, v=None, g=9.81, s=0.0):
        L = _lib.load()
        if not isinstance(system, GPUCellList):
            raise TypeError("system must be a GPUCellList")
        D, N = system.dim, system.n
        if sphkernel is not None and getattr(sphkernel, "dim", D) != D:
            raise ValueError("kernel dimension does not match the cell list")
        if int(gamma) != gamma or int(gamma) <= 0:
            raise ValueError("gamma must be a positive integer (Float64^Int equation of state)")
        self.system = system
        self.dim = D
        self.sphkernel = sphkernel if sphkernel is not None else WendlandC2(dim=D)
        self.rho = _cuda_f64(rho, N, "ρ")
        pt = torch.as_tensor(ptype)
        if pt.numel() != N:
            raise ValueError(f"length(ptype) ({pt.numel()}) != N ({N})")
        self.ptype = pt.to(device="cuda", dtype=torch.int32).contiguous()
        if v is None:
            self.v = tuple(torch.zeros(N, dtype=torch.float64, device="cuda") for _ in range(D))
        else:
            if len(v) != D:
                raise ValueError(f"length(v) ({len(v)}) != dim ({D})")
            self.v = tuple(_cuda_f64(vi, N, "v") for vi in v)
        p = _lib.gcsph_params()
        p.dx, p.h, p.H = float(dx), float(h), float(H)
        p.rho0, p.m0, p.dt, p.alpha = float(rho0), float(m0), float(dt), float(alpha)
        p.nu, p.g, p.c0, p.s, p.delta, p.CFL = 0.0, float(g), float(c0), float(s), float(delta), float(CFL)
        p.nui = system.dist - float(H)
        p.etime = 0.0
        p.dpc_l0, p.dpc_pmin, p.dpc_pmax, p.dpc_lambda = 0.0, 1.0, 10000.0, 0.01
        p.xsph_eps = 0.0
        p.bound_D, p.bound_l = 0.4, 2 * float(dx)
        p.gamma, p.cspmn = int(gamma), 15
        h_ = C.c_void_p()
        _lib.check(L.sph_create(system._h, C.byref(p), _lib.dptr(self.rho), _lib.ptrs(self.v),
                                _lib.dptr(self.ptype), C.byref(h_)))
        self._h = h_
        self.h_inv = 1.0 / float(h)
        self.H_inv = 1.0 / float(H)

    # --------------------------------------------------------------- scalar fields
    def _params(self):
        p = _lib.gcsph_params()
        _lib.check(_lib.load().sph_get_params(self._h, C.byref(p)))
        return p

    def __getattr__(self, name):
        if name in _PARAM_FIELDS and "_h" in self.__dict__:
            return getattr(self._params(), name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in _PARAM_FIELDS and "_h" in self.__dict__:
            p = self._params()
            setattr(p, name, int(value) if name in ("gamma", "cspmn") else float(value))
            _lib.check(_lib.load().sph_set_params(self._h, C.byref(p)))
        else:
            object.__setattr__(self, name, value)

    def set_lanes(self, lanes: int):
        """Lanes per particle in the pair passes (0 = auto, 1 = serial row
        order, bit-identical to the CPU oracle)."""
        _lib.check(_lib.load().sph_set_lanes(self._h, int(lanes)))

    def set_graphs(self, on: bool):
        """Run stepsolve! calls as captured CUDA graphs where update! follows
        every step (default on); off runs one host round trip per step."""
        _lib.check(_lib.load().sph_set_graphs(self._h, int(bool(on))))

    def set_dt_variant(self, relative: bool):
        """Δt_stepping's velocity term: False (default) as the reference writes
        it (absolute v·x per particle), True the pair-relative bound
        max |h Δv·Δx / (|Δx|² + η²)|."""
        _lib.check(_lib.load().sph_set_dt_variant(self._h, int(bool(relative))))

    def graph_stats(self):
        """(graphs captured, calls replayed as a graph) so far."""
        a, b = C.c_int64(), C.c_int64()
        _lib.check(_lib.load().sph_graph_stats(self._h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    # --------------------------------------------------------------- fields
    def field(self, name: str):
        """Copy of one library field in original particle order."""
        D, N = self.dim, self.system.n
        if name in _lib.VECTOR_FIELDS:
            out = torch.empty((D, N), dtype=torch.float64, device="cuda")
        elif name == "ptype":
            out = torch.empty(N, dtype=torch.int32, device="cuda")
        else:
            out = torch.empty(N, dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().sph_get_field(self._h, _lib.FIELDS[name], _lib.dptr(out)))
        return tuple(out[d] for d in range(D)) if name in _lib.VECTOR_FIELDS else out

    # --------------------------------------------------------------- stepping
    def stepsolve(self, n: int = 1, timestepping: bool = False, timelims=None):
        """stepsolve!(prob, n; timestepping, timelims) -- src/sphproblem.jl:204-345.

        Returns (updaten, maxcΔxout).  The default timelims are
        (sqrt(eps()), CFL*H/3c₀) as in _stepsolve! (:207)."""
        if timelims is None:
            timelims = (math.sqrt(_EPS), self.CFL * self.H / (3 * self.c0))
        un = C.c_int64()
        mc = C.c_double()
        prev = self.system.pairsn
        _lib.check(_lib.load().sph_step(self._h, int(n), int(bool(timestepping)), float(timelims[0]),
                                        float(timelims[1]), C.byref(un), C.byref(mc)))
        if un.value > 0:
            # update! ran inside: refresh the cell list's user-visible fields
            self.system._refresh_cellpnum()
            tot = C.c_int64()
            _lib.load().gcl_emit_pairs(self.system._h, None, 0, 0, C.byref(tot))
            self.system._apply_update_policy(prev, int(tot.value), True)
        return int(un.value), float(mc.value)

    def close(self):
        h = self.__dict__.get("_h")
        if h:
            _lib.load().sph_destroy(h)
            object.__setattr__(self, "_h", None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __repr__(self):
        s = f"  SPH Problem \n{self.system!r}\n  h: {self.h}\n  H: {self.H}\n  SPH Kernel: {self.sphkernel!r}\n"
        s += f"  E Time: {self.etime}\n"
        s += f"  Surface tension: {self.s}\n" if self.s > 0 else "  Surface tension: not used\n"
        if self.dpc_l0 > 0 and self.dpc_lambda > 0:
            s += f"  DPC: l₀ = {self.dpc_l0} , λ = {self.dpc_lambda}\n"
        else:
            s += "  DPC: not used\n"
        return s


def stepsolve(prob: SPHProblem, n: int = 1, timestepping: bool = False, timelims=None):
    return prob.stepsolve(n, timestepping=timestepping, timelims=timelims)


# getters, src/sphproblem.jl:348-390
def get_points(prob: SPHProblem):
    return prob.system.points


def get_velocity(prob: SPHProblem):
    return prob.v


def get_density(prob: SPHProblem):
    return prob.rho


def get_pressure(prob: SPHProblem):
    return prob.field("P")


def get_acceleration(prob: SPHProblem):
    return prob.field("a")


def get_dpccorr(prob: SPHProblem):
    return prob.field("buf2")


def get_simtime(prob: SPHProblem):
    return prob.etime


def get_dt(prob: SPHProblem):
    return prob.dt


def get_sumw(prob: SPHProblem):
    return prob.field("sumW")


def get_sumgradw(prob: SPHProblem):
    return prob.field("sumgW")


def get_ptype(prob: SPHProblem):
    return prob.ptype


def timesolve(prob: SPHProblem, batch: int = 10, timeframe: float = 1.0, writetime: float = 0, path=None,
              pvc: bool = False, vtkvars=("Acceleration", "Velocity", "Pressure"), timestepping: bool = False,
              timelims=None, anim: bool = False, verbose: bool = True, callback=None):
    """timesolve!(prob; batch, timeframe, ...) -- src/sphproblem.jl:420-511.

    Runs stepsolve(prob, batch) while etime <= timeframe.  With `path` and
    writetime > 0 it writes OUTPUT_<i>.vtp frames of `vtkvars` every
    `writetime` of simulated time (and OUTPUT_PVC.pvd with pvc=True), as the
    reference does; the frames are copied into pinned host memory after the
    batch that produced them and written by a background thread while the
    next batches run.  `callback(prob, i)` is called at the same moments.
    `anim` is not supported (no graphics stack)."""
    from . import vtkio
    lim = prob.CFL * prob.H / (3 * prob.c0)
    if timelims is None:
        timelims = (math.sqrt(_EPS), lim)
    if timelims[1] > lim:
        warnings.warn(f"Maximum dt limit ({timelims[1]}) > CFL*H/3c₀ ({lim})")
    if timestepping:
        timelims = (max(timelims[0], _EPS), min(timelims[1], lim))
    if anim:
        raise NotImplementedError("animation needs a graphics stack; write frames with `path` or `callback`")
    if verbose:
        print("    Start simulation...")
        print(f"Timestepping: {timestepping}")
        if timestepping:
            print(f"Δt limitss: {timelims}")
        print(f"Batch: {batch}")
        print(f"NUI: {prob.nui}")
    nt = prob.etime + writetime
    i = 0
    writer = vtkio.AsyncWriter(path, pvc=pvc) if (writetime > 0 and path is not None) else None

    def frame(k):
        if writer is not None:
            writer.submit(f"OUTPUT_{k:05d}", vtkio.Snapshot(prob, vtkvars))
        if callback is not None:
            callback(prob, k)

    if writetime > 0:
        frame(i)
    diag = (0, 0.0)
    t0 = time.perf_counter()
    try:
        while prob.etime <= timeframe:
            diag = prob.stepsolve(batch, timestepping=timestepping, timelims=timelims)
            if writetime > 0 and nt < prob.etime:
                nt += writetime
                frame(i)
            i += 1
    finally:
        if writer is not None:
            writer.close()
    if verbose:
        print(f"iter: {i}, time: {prob.etime}, Δt: {prob.dt}, updn: {diag[0]}, dxpncu: {diag[1]}, "
              f"wall: {time.perf_counter() - t0:.3f}s")
    return diag
