"""CPU-side checks of the C ABI: the library builds, loads without a GPU and
exports every function include/gcsph.h declares; host-only entry points agree
with the oracle."""
import ctypes as C
import os
import re

from conftest import ROOT


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "gcsph.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"\{[^{}]*\}", "", src)  # struct and enum bodies (callback members are not exports)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(\w+)\s*\(", src, flags=re.M)
    return sorted({n for n in names if n not in ("if", "defined")})


def test_library_exports_every_declared_symbol(pkg):
    L = pkg.load_library()
    declared = _declared_functions()
    assert len(declared) >= 40
    missing = [n for n in declared if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding covers each of them
    from importlib import import_module
    lib_mod = import_module(pkg.__name__ + "._lib")
    assert set(declared) <= set(lib_mod.symbols()), set(declared) - set(lib_mod.symbols())


def test_host_only_entry_points(pkg, orc):
    L = pkg.load_library()
    assert L.gcsph_version() == 1
    for D in (2, 3):
        assert L.gcsph_dpckernlim(D) == orc.lib().orc_dpckernlim(D)
    n0 = L.gcsph_launch_count()
    assert isinstance(n0, int)


def test_error_path_without_gpu(pkg):
    """Invalid arguments fail with a status code and a message, no crash."""
    L = pkg.load_library()
    h = C.c_void_p()
    rc = L.gcl_create(4, 10, None, None, 0.1, None, None, None, C.byref(h))
    assert rc == 1
    assert b"null" in L.gcsph_last_error() or b"dimention" in L.gcsph_last_error()
