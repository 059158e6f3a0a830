"""ctypes binding of libgcsph.so (include/gcsph.h).

There is no CPU fallback: if the CUDA library cannot be built or loaded, every
call raises.  Device pointers come from CUDA torch tensors (data_ptr()).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

GCSPH_OK, GCSPH_EINVAL, GCSPH_ECAPACITY, GCSPH_ECUDA, GCSPH_ENOMEM, GCSPH_ESTATE = range(6)

FIELDS = {"x": 0, "rho": 1, "v": 2, "P": 3, "a": 4, "drhodt": 5, "rhoh": 6, "vh": 7, "xh": 8, "cdx": 9,
          "sumW": 10, "sumgW": 11, "buf2": 12, "ptype": 13}
VECTOR_FIELDS = {"x", "v", "a", "vh", "xh", "cdx", "sumgW", "buf2"}


class GcsphError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gcsph error {code}: {msg}")
        self.code = code


class gcsph_params(C.Structure):
    """Mirror of gcsph_params (mutable SPHProblem scalars)."""
    _fields_ = [(n, C.c_double) for n in (
        "dx", "h", "H", "rho0", "m0", "dt", "alpha", "nu", "g", "c0", "s", "delta", "CFL", "nui", "etime",
        "dpc_l0", "dpc_pmin", "dpc_pmax", "dpc_lambda", "xsph_eps", "bound_D", "bound_l")] + [
        ("gamma", C.c_int32), ("cspmn", C.c_int32)]


class gcsph_ens_params(C.Structure):
    """Mirror of gcsph_ens_params (one ensemble instance)."""
    _fields_ = [(n, C.c_double) for n in (
        "dx", "h", "H", "rho0", "m0", "dt", "alpha", "nu", "g", "c0", "s", "delta", "bound_D", "bound_l")] + [
        ("grid_min", C.c_double * 3), ("grid_max", C.c_double * 3)] + [
        (n, C.c_double) for n in ("dpc_l0", "dpc_pmin", "dpc_pmax", "dpc_lambda", "xsph_eps")] + [
        ("gamma", C.c_int32), ("cspmn", C.c_int32)]


ENS_FIELDS = {"x": 0, "v": 1, "rho": 2, "P": 3, "ptype": 4, "drho": 5}

vp = C.c_void_p
i32, i64, f64 = C.c_int32, C.c_int64, C.c_double
PP = C.POINTER(C.c_void_p)  # host array of device pointers

# serving scheduler: backend callbacks and statistics (mirrors of gcsph.h)
SRV_ADD = C.CFUNCTYPE(C.c_int, vp, i32, i32, C.POINTER(i32))
SRV_REMOVE = C.CFUNCTYPE(C.c_int, vp, i32, i32)
SRV_STEP = C.CFUNCTYPE(C.c_int, vp, i32, i32)
SRV_HARVEST = C.CFUNCTYPE(C.c_int, vp, i32, i32, i32)
SRV_FREE = C.CFUNCTYPE(i64, vp)
SRV_BPP = C.CFUNCTYPE(i64, vp, i32)
SRV_NOW = C.CFUNCTYPE(f64, vp)


class gcsph_srv_backend(C.Structure):
    _fields_ = [("ctx", vp), ("add", SRV_ADD), ("remove", SRV_REMOVE), ("step", SRV_STEP), ("harvest", SRV_HARVEST),
                ("free_bytes", SRV_FREE), ("bytes_per_particle", SRV_BPP), ("now", SRV_NOW)]


class gcsph_srv_stats(C.Structure):
    _fields_ = [("requests", i32), ("completed", i32), ("particle_steps", i64), ("wall_s", f64), ("p50_s", f64),
                ("p99_s", f64), ("mean_s", f64)]


_SIGS = {
    "gcsph_last_error": (C.c_char_p, []),
    "gcsph_version": (C.c_int, []),
    "gcsph_launch_count": (C.c_uint64, []),
    "gcsph_timing_enable": (C.c_int, [C.c_int]),
    "gcsph_timing_reset": (C.c_int, []),
    "gcsph_timing_count": (C.c_int, []),
    "gcsph_timing_name": (C.c_char_p, [i32]),
    "gcsph_timing_get": (C.c_int, [i32, C.POINTER(i64), C.POINTER(f64)]),
    "gcl_create": (C.c_int, [i32, i64, PP, C.POINTER(f64), f64, C.POINTER(f64), C.POINTER(f64), vp, C.POINTER(vp)]),
    "gcl_destroy": (None, [vp]),
    "gcl_grid": (C.c_int, [vp, C.POINTER(f64), C.POINTER(f64), C.POINTER(i64)]),
    "gcl_update": (C.c_int, [vp, C.POINTER(i64)]),
    "gcl_partialupdate": (C.c_int, [vp, C.POINTER(i64)]),
    "gcl_emit_pairs": (C.c_int, [vp, vp, i64, C.c_int, C.POINTER(i64)]),
    "gcl_cellpnum": (C.c_int, [vp, vp]),
    "gcl_maxpairs": (C.c_int, [vp, C.POINTER(i64)]),
    "gcl_set_sort": (C.c_int, [vp, i32]),
    "gcl_pairs_noalloc": (C.c_int, [i32, i64, PP, C.POINTER(f64), f64, C.POINTER(f64), C.POINTER(f64), vp, i64,
                                    C.c_int, C.POINTER(i64), vp]),
    "gcl_pairs_noalloc_init": (C.c_int, []),
    "sph_create": (C.c_int, [vp, C.POINTER(gcsph_params), vp, PP, vp, C.POINTER(vp)]),
    "sph_destroy": (None, [vp]),
    "sph_set_params": (C.c_int, [vp, C.POINTER(gcsph_params)]),
    "sph_get_params": (C.c_int, [vp, C.POINTER(gcsph_params)]),
    "sph_set_lanes": (C.c_int, [vp, i32]),
    "sph_set_graphs": (C.c_int, [vp, i32]),
    "sph_set_dt_variant": (C.c_int, [vp, i32]),
    "sph_graph_stats": (C.c_int, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "sph_step": (C.c_int, [vp, i32, C.c_int, f64, f64, C.POINTER(i64), C.POINTER(f64)]),
    "ens_create": (C.c_int, [i32, vp, C.POINTER(vp)]),
    "ens_destroy": (None, [vp]),
    "ens_bytes_per_particle": (C.c_int, [i32, C.POINTER(i64)]),
    "ens_add": (C.c_int, [vp, i64, vp, vp, vp, vp, C.POINTER(gcsph_ens_params), C.POINTER(i32)]),
    "ens_remove": (C.c_int, [vp, i32]),
    "ens_step": (C.c_int, [vp, i32]),
    "ens_set_stream": (C.c_int, [vp, vp]),
    "ens_get": (C.c_int, [vp, i32, i32, vp]),
    "ens_info": (C.c_int, [vp, i32, C.POINTER(i64), C.POINTER(i64), C.POINTER(f64)]),
    "ens_totals": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i64), C.POINTER(i64)]),
    "ens_set_tuning": (C.c_int, [vp, i32, i32]),
    "ens_get_tuning": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i64), C.POINTER(i64)]),
    "ens_set_list_build": (C.c_int, [vp, i32, i32, i32, i32]),
    "ens_set_skin": (C.c_int, [vp, C.c_double]),
    "ens_get_skin": (C.c_int, [vp, C.POINTER(C.c_double)]),
    "ens_list_builds": (C.c_int, [vp, i32, C.POINTER(i64)]),
    "ens_set_dpc_bound": (C.c_int, [vp, i32]),
    "ens_get_dpc_bound": (C.c_int, [vp, C.POINTER(i32)]),
    "ens_get_list_build": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
    "srv_create": (C.c_int, [vp, i32, f64, C.c_uint32, C.POINTER(gcsph_srv_backend), C.POINTER(vp)]),
    "srv_destroy": (None, [vp]),
    "srv_submit": (C.c_int, [vp, i32, i64, vp, vp, vp, vp, C.POINTER(gcsph_ens_params), i64, f64, C.POINTER(i32)]),
    "srv_progress": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32)]),
    "srv_run": (C.c_int, [vp]),
    "srv_set_policy": (C.c_int, [vp, i32, i64, i64, f64]),
    "srv_get_policy": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i64), C.POINTER(i64), C.POINTER(f64)]),
    "srv_request": (C.c_int, [vp, i32, C.POINTER(i32), C.POINTER(f64), C.POINTER(f64), C.POINTER(f64)]),
    "srv_result": (C.c_int, [vp, i32, i32, vp]),
    "srv_stats": (C.c_int, [vp, C.POINTER(gcsph_srv_stats)]),
    "ens_set_list_stride": (C.c_int, [vp, i32]),
    "ens_get_list_stride": (C.c_int, [vp, C.POINTER(i32)]),
    "sph_get_field": (C.c_int, [vp, i32, vp]),
    "gcsph_dpckernlim": (f64, [i32]),
    "gcsph_sphW": (C.c_int, [i32, i64, i64, vp, PP, f64, vp, vp]),
    "gcsph_sphgradW": (C.c_int, [i32, i64, i64, vp, PP, f64, PP, vp]),
    "gcsph_sphsumW": (C.c_int, [i32, i64, i64, vp, PP, f64, vp, vp, vp]),
    "gcsph_sphsumgradW": (C.c_int, [i32, i64, i64, vp, PP, f64, vp, PP, vp]),
    "gcsph_drhodt_ddt": (C.c_int, [i32, i64, i64, vp, PP, vp, PP, PP, f64, f64, f64, f64, i32, f64, f64, vp, vp, vp]),
    "gcsph_pressure": (C.c_int, [i64, vp, f64, i32, f64, vp, vp, vp]),
    "gcsph_dvdt": (C.c_int, [i32, i64, i64, vp, PP, vp, f64, vp, vp, PP, vp]),
    "gcsph_dvdt_av": (C.c_int, [i32, i64, i64, vp, PP, PP, f64, vp, f64, PP, f64, f64, vp, PP, vp]),
    "gcsph_dvdt_visc": (C.c_int, [i32, i64, i64, vp, PP, PP, vp, PP, f64, f64, f64, vp, PP, vp]),
    "gcsph_addgrav": (C.c_int, [i32, i64, f64, PP, vp]),
    "gcsph_fbmolforce": (C.c_int, [i32, i64, i64, vp, PP, f64, f64, vp, PP, vp]),
    "gcsph_dvdt_pF": (C.c_int, [i32, i64, i64, vp, PP, f64, f64, f64, vp, PP, vp]),
    "gcsph_update_rho": (C.c_int, [i64, vp, vp, f64, f64, vp, vp]),
    "gcsph_update_v": (C.c_int, [i32, i64, PP, PP, f64, vp, vp]),
    "gcsph_update_x": (C.c_int, [i32, i64, PP, PP, f64, vp]),
    "gcsph_symplectic": (C.c_int, [i32, i64, vp, vp, PP, PP, PP, PP, vp, PP, f64, PP, f64, vp, vp]),
    "gcsph_dpcreg": (C.c_int, [i32, i64, i64, PP, PP, vp, vp, vp, PP, f64, f64, f64, f64, f64, f64, vp, vp]),
    "gcsph_update_dpcreg": (C.c_int, [i32, i64, PP, PP, PP, f64, vp, vp]),
    "gcsph_xsphcorr": (C.c_int, [i32, i64, i64, PP, vp, vp, vp, PP, f64, f64, vp, vp]),
    "gcsph_update_xsph": (C.c_int, [i32, i64, PP, PP, f64, vp, vp]),
    "gcsph_cspmcorr": (C.c_int, [i32, i64, i64, PP, vp, vp, f64, vp, vp, vp]),
    "gcsph_dt_stepping": (C.c_int, [i32, i64, PP, PP, PP, f64, f64, f64, f64, f64, C.POINTER(f64), vp]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building if needed) libgcsph.so and bind every exported symbol."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path) or not _build.up_to_date():
            if not build_if_missing:
                raise OSError(f"libgcsph.so not built at {path}")
            _build.build()
        L = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return _lib


def symbols():
    return list(_SIGS)


def check(rc: int, allow=()):
    if rc != GCSPH_OK and rc not in allow:
        msg = load().gcsph_last_error()
        raise GcsphError(rc, msg.decode() if msg else "")
    return rc


def ptrs(tensors):
    """Host array of device pointers for a tuple of tensors (or None)."""
    if tensors is None:
        return None
    arr = (C.c_void_p * 3)()
    for d, t in enumerate(tensors):
        arr[d] = t.data_ptr() if t is not None else None
    return C.cast(arr, PP)


def dptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def launch_count() -> int:
    return int(load().gcsph_launch_count())
