"""ctypes binding of the CPU oracle (oracle/gcsph_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker or the timed CPU
baseline, never as the product path.  Parity of this oracle against the
reference's own outputs is UNPINNED (the reference is GPU-only Julia and
ships no expected values); the pair set is pinned by an O(N^2) brute force.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# the parity build (-O2) that the tests check against, and the same source
# at -O3 that the benchmark times as the CPU baseline (oracle/Makefile)
_BUILDS = {"parity": os.path.join(_HERE, "_build", "liboracle.so"),
           "timed": os.path.join(_HERE, "_build", "liboracle_timed.so")}
_LIB_PATH = _BUILDS["parity"]
_lib = None


def select_build(name: str) -> None:
    """Choose which build lib() loads: "parity" (default) or "timed".  Must
    come before the first lib() call of the process."""
    global _LIB_PATH
    path = _BUILDS[name]
    if _lib is not None and path != _LIB_PATH:
        raise RuntimeError(f"oracle: the {_LIB_PATH} build is already loaded")
    _LIB_PATH = path


def loaded_build() -> str:
    """The file name of the build lib() loads."""
    return os.path.basename(_LIB_PATH)

f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class OrcParams(C.Structure):
    """Mutable SPHProblem fields (src/sphproblem.jl:62-112)."""
    _fields_ = [(n, C.c_double) for n in (
        "dx", "h", "H", "rho0", "m0", "dt", "alpha", "nu", "g", "c0", "s", "delta", "CFL", "nui",
        "etime", "dpc_l0", "dpc_pmin", "dpc_pmax", "dpc_lambda", "xsph_eps", "bound_D", "bound_l")] + [
        ("gamma", C.c_int32), ("cspmn", C.c_int32)]


FIELDS = {"x": 0, "rho": 1, "v": 2, "P": 3, "a": 4, "drhodt": 5, "rhoh": 6, "vh": 7, "xh": 8,
          "cdx": 9, "sumW": 10, "sumgW": 11, "buf2": 12, "ptype": 13}
VECTOR_FIELDS = {"x", "v", "a", "vh", "xh", "cdx", "sumgW", "buf2"}


def build() -> str:
    """Compile liboracle.so with its Makefile (portable flags only)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_max_threads.restype = C.c_int
        L.orc_wendland_w.restype = C.c_double
        L.orc_wendland_w.argtypes = [C.c_int, C.c_double, C.c_double]
        L.orc_wendland_dw.restype = C.c_double
        L.orc_wendland_dw.argtypes = [C.c_int, C.c_double, C.c_double]
        L.orc_powfancy7th.restype = C.c_double
        L.orc_powfancy7th.argtypes = [C.c_double, C.c_double, C.c_int32]
        L.orc_ipow.restype = C.c_double
        L.orc_ipow.argtypes = [C.c_double, C.c_int32]
        L.orc_dpckernlim.restype = C.c_double
        L.orc_dpckernlim.argtypes = [C.c_int]
        L.orc_grid.restype = C.c_int
        L.orc_grid.argtypes = [C.c_int, C.c_int64, f64p, f64p, C.c_double, C.c_void_p, C.c_void_p,
                               f64p, f64p, i64p]
        L.orc_cellmap.argtypes = [C.c_int, C.c_int64, f64p, f64p, f64p, i64p, i32p, i32p]
        L.orc_maxpairs.restype = C.c_int64
        L.orc_maxpairs.argtypes = [C.c_int, i32p, i64p]
        L.orc_neib_search.restype = C.c_int64
        L.orc_neib_search.argtypes = [C.c_int, C.c_int64, f64p, i32p, i64p, C.c_double, i32p, C.c_int64]
        L.orc_pairs_bruteforce.restype = C.c_int64
        L.orc_pairs_bruteforce.argtypes = [C.c_int, C.c_int64, f64p, i32p, C.c_double, i32p, C.c_int64]
        L.orc_sys_create.restype = C.c_void_p
        L.orc_sys_create.argtypes = [C.c_int, C.c_int64, f64p, f64p, C.c_double, f64p, C.c_void_p, i32p,
                                     C.POINTER(OrcParams)]
        L.orc_sys_destroy.argtypes = [C.c_void_p]
        L.orc_sys_set_params.argtypes = [C.c_void_p, C.POINTER(OrcParams)]
        L.orc_sys_get_params.argtypes = [C.c_void_p, C.POINTER(OrcParams)]
        L.orc_sys_stepsolve.argtypes = [C.c_void_p, C.c_int32, C.c_int, C.c_double, C.c_double,
                                        C.POINTER(C.c_int64), C.POINTER(C.c_double)]
        L.orc_sys_get.restype = C.c_int
        L.orc_sys_get.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_sys_pairsn.restype = C.c_int64
        L.orc_sys_pairsn.argtypes = [C.c_void_p]
        L.orc_sys_paircap.restype = C.c_int64
        L.orc_sys_paircap.argtypes = [C.c_void_p]
        L.orc_sys_pairs.argtypes = [C.c_void_p, i32p]
        L.orc_sys_grid.argtypes = [C.c_void_p, f64p, f64p, i64p]
        L.orc_sys_partialupdate.argtypes = [C.c_void_p, C.c_int]
        L.orc_sys_update.argtypes = [C.c_void_p]
        L.orc_sys_set_x.argtypes = [C.c_void_p, f64p]
        L.orc_sys_set_xh.argtypes = [C.c_void_p, f64p]
        I, N64, P64, D64 = C.c_int, C.c_int64, C.c_int64, C.c_double
        vpp = C.c_void_p
        sigs = {
            "orc_sphW": [I, N64, P64, vpp, vpp, D64, vpp],
            "orc_sphgradW": [I, N64, P64, vpp, vpp, D64, vpp],
            "orc_sphsumW": [I, N64, P64, vpp, vpp, D64, vpp, vpp],
            "orc_sphsumgradW": [I, N64, P64, vpp, vpp, D64, vpp, vpp],
            "orc_drhodt_ddt": [I, N64, P64, vpp, vpp, vpp, vpp, vpp, D64, D64, D64, D64, C.c_int32, D64, D64, vpp,
                               vpp],
            "orc_pressure": [N64, vpp, D64, C.c_int32, D64, vpp, vpp],
            "orc_dvdt": [I, N64, P64, vpp, vpp, vpp, D64, vpp, vpp, vpp],
            "orc_dvdt_av": [I, N64, P64, vpp, vpp, vpp, D64, vpp, D64, vpp, D64, D64, vpp, vpp],
            "orc_dvdt_visc": [I, N64, P64, vpp, vpp, vpp, vpp, vpp, D64, D64, D64, vpp, vpp],
            "orc_addgrav": [I, N64, D64, vpp],
            "orc_fbmolforce": [I, N64, P64, vpp, vpp, D64, D64, vpp, vpp],
            "orc_dvdt_pF": [I, N64, P64, vpp, vpp, D64, D64, D64, vpp, vpp],
            "orc_update_rho": [N64, vpp, vpp, D64, D64, vpp],
            "orc_update_v": [I, N64, vpp, vpp, D64, vpp],
            "orc_update_x": [I, N64, vpp, vpp, D64],
            "orc_symplectic": [I, N64, vpp, vpp, vpp, vpp, vpp, vpp, vpp, vpp, D64, vpp, D64, vpp],
            "orc_dpcreg": [I, N64, P64, vpp, vpp, vpp, vpp, vpp, vpp, D64, D64, D64, D64, D64, D64, vpp],
            "orc_update_dpcreg": [I, N64, vpp, vpp, vpp, D64, vpp],
            "orc_xsphcorr": [I, N64, P64, vpp, vpp, vpp, vpp, vpp, D64, D64, vpp],
            "orc_update_xsph": [I, N64, vpp, vpp, D64, vpp],
            "orc_cspmcorr": [I, N64, P64, vpp, vpp, vpp, D64, vpp, vpp],
            "orc_dt_stepping": [I, N64, vpp, vpp, vpp, D64, D64, D64, D64, D64],
        }
        for name, args in sigs.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = None
        L.orc_dt_stepping.restype = C.c_double
        _lib = L
    return _lib


def call(name, *args):
    """Call a per-function oracle routine; numpy arrays are passed by pointer."""
    conv = [a.ctypes.data if isinstance(a, np.ndarray) else a for a in args]
    return getattr(lib(), name)(*conv)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


# ---------------------------------------------------------------- cell list
def grid(x: np.ndarray, cellsize, dist, MIN=None, MAX=None):
    """Grid of GPUCellList (src/celllist.jl:27-46). x is (D, N) float64."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    D, N = x.shape
    cs = np.zeros(D); off = np.zeros(D); cell = np.zeros(D, dtype=np.int64)
    mn = None if MIN is None else np.ascontiguousarray(MIN, dtype=np.float64)
    mx = None if MAX is None else np.ascontiguousarray(MAX, dtype=np.float64)
    rc = lib().orc_grid(D, N, x, np.ascontiguousarray(cellsize, dtype=np.float64), float(dist),
                        None if mn is None else mn.ctypes.data, None if mx is None else mx.ctypes.data,
                        cs, off, cell)
    if rc != 0:
        raise ValueError("degenerate grid")
    return cs, off, cell


def cellmap(x, cs, off, cell):
    x = np.ascontiguousarray(x, dtype=np.float64)
    D, N = x.shape
    pcell = np.zeros((D, N), dtype=np.int32)
    cellpnum = np.zeros(int(np.prod(cell)), dtype=np.int32)
    lib().orc_cellmap(D, N, x, np.asarray(cs, np.float64), np.asarray(off, np.float64),
                      np.asarray(cell, np.int64), pcell, cellpnum)
    return pcell, cellpnum


def maxpairs(D, cellpnum, cell) -> int:
    return int(lib().orc_maxpairs(D, np.ascontiguousarray(cellpnum, np.int32), np.asarray(cell, np.int64)))


def neib_search(x, pcell, cell, dist, cap=None):
    """Pair list by the reference's cell-list algorithm. Returns (pairs[n,2], total)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    D, N = x.shape
    L = lib()
    if cap is None:
        cap = int(L.orc_neib_search(D, N, x, np.ascontiguousarray(pcell, np.int32),
                                    np.asarray(cell, np.int64), float(dist), np.zeros(2, np.int32), 0))
    out = np.zeros(2 * max(cap, 1), dtype=np.int32)
    n = int(L.orc_neib_search(D, N, x, np.ascontiguousarray(pcell, np.int32), np.asarray(cell, np.int64),
                              float(dist), out, cap))
    return out.reshape(-1, 2)[:min(n, cap)], n


def pairs_bruteforce(x, pcell, dist):
    x = np.ascontiguousarray(x, dtype=np.float64)
    D, N = x.shape
    L = lib()
    n = int(L.orc_pairs_bruteforce(D, N, x, np.ascontiguousarray(pcell, np.int32), float(dist),
                                   np.zeros(2, np.int32), 0))
    out = np.zeros(2 * max(n, 1), dtype=np.int32)
    L.orc_pairs_bruteforce(D, N, x, np.ascontiguousarray(pcell, np.int32), float(dist), out, n)
    return out.reshape(-1, 2)[:n]


def pair_set(pairs: np.ndarray) -> np.ndarray:
    """Canonical sorted (n,2) view of a pair list (rows with first index 0 dropped)."""
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    p = p[p[:, 0] != 0]
    key = p[:, 0] * (1 << 32) + p[:, 1]
    return p[np.argsort(key, kind="stable")]


# ---------------------------------------------------------------- full problem
def default_params(dx, h, H, rho0, m0, dt, alpha, c0, gamma, delta, CFL, dist, g=9.81, s=0.0) -> OrcParams:
    """SPHProblem constructor defaults, src/sphproblem.jl:147-191."""
    return OrcParams(dx=dx, h=h, H=H, rho0=rho0, m0=m0, dt=dt, alpha=alpha, nu=0.0, g=g, c0=c0, s=s,
                     delta=delta, CFL=CFL, nui=dist - H, etime=0.0, dpc_l0=0.0, dpc_pmin=1.0,
                     dpc_pmax=10000.0, dpc_lambda=0.01, xsph_eps=0.0, bound_D=0.4, bound_l=2 * dx,
                     gamma=int(gamma), cspmn=15)


class OracleSystem:
    """GPUCellList + SPHProblem + stepsolve! on the CPU (original particle order)."""

    def __init__(self, x, cellsize, dist, rho, ptype, params: OrcParams, v=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        self.D, self.N = x.shape
        self.dist = float(dist)
        L = lib()
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        self._h = L.orc_sys_create(self.D, self.N, x, np.ascontiguousarray(cellsize, np.float64), float(dist),
                                   np.ascontiguousarray(rho, np.float64),
                                   None if vv is None else vv.ctypes.data,
                                   np.ascontiguousarray(ptype, np.int32), C.byref(params))
        if not self._h:
            raise ValueError("oracle: degenerate grid")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_sys_destroy(self._h)
            self._h = None

    @property
    def params(self) -> OrcParams:
        p = OrcParams()
        lib().orc_sys_get_params(self._h, C.byref(p))
        return p

    @params.setter
    def params(self, p: OrcParams):
        lib().orc_sys_set_params(self._h, C.byref(p))

    def stepsolve(self, n=1, timestepping=False, timelims=None):
        p = self.params
        if timelims is None:
            timelims = (np.sqrt(np.finfo(np.float64).eps), p.CFL * p.H / (3 * p.c0))
        un = C.c_int64(0); mc = C.c_double(0)
        lib().orc_sys_stepsolve(self._h, int(n), int(bool(timestepping)), float(timelims[0]),
                                float(timelims[1]), C.byref(un), C.byref(mc))
        return int(un.value), float(mc.value)

    def get(self, name):
        shape = (self.D, self.N) if name in VECTOR_FIELDS else (self.N,)
        out = np.zeros(shape, dtype=np.int32 if name == "ptype" else np.float64)
        rc = lib().orc_sys_get(self._h, FIELDS[name], out.ctypes.data)
        assert rc == 0
        return out

    @property
    def pairsn(self) -> int:
        return int(lib().orc_sys_pairsn(self._h))

    def pairs(self) -> np.ndarray:
        cap = int(lib().orc_sys_paircap(self._h))
        out = np.zeros(2 * max(cap, 1), dtype=np.int32)
        lib().orc_sys_pairs(self._h, out)
        return out.reshape(-1, 2)[:cap]

    def grid(self):
        cs = np.zeros(self.D); off = np.zeros(self.D); cell = np.zeros(self.D, np.int64)
        lib().orc_sys_grid(self._h, cs, off, cell)
        return cs, off, cell

    def update(self):
        lib().orc_sys_update(self._h)

    def partialupdate(self, fillzero=True):
        lib().orc_sys_partialupdate(self._h, int(bool(fillzero)))

    def set_x(self, x):
        lib().orc_sys_set_x(self._h, np.ascontiguousarray(x, dtype=np.float64))

    def set_xh(self, x):
        lib().orc_sys_set_xh(self._h, np.ascontiguousarray(x, dtype=np.float64))
