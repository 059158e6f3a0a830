"""gcl_pairs_noalloc: the pair list in one call that allocates no device memory.

It exists for callers that may not allocate device memory while they run (a
process whose own pool already holds the GPU, a plugin host that forbids it,
a time-critical loop that cannot absorb cudaMalloc's implicit synchronisation).
This file is collected last so that a failure here stops a `-x` run only
after every other test has run; it also passes on its own in a fresh process.
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from conftest import ROOT

pytestmark = pytest.mark.gpu


def _noalloc(L, x, cs, dist, cap, fillzero=1):
    D, N = x.shape
    xs = tuple(torch.from_numpy(np.ascontiguousarray(x[d])).cuda() for d in range(D))
    ptrs = (C.c_void_p * 3)(*[t.data_ptr() for t in xs])
    out = torch.full((max(cap, 1), 2), -7, dtype=torch.int32, device="cuda")
    n = C.c_int64()
    rc = L.gcl_pairs_noalloc(D, N, C.cast(ptrs, C.POINTER(C.c_void_p)), (C.c_double * 3)(*cs), float(dist), None,
                             None, C.c_void_p(out.data_ptr()), cap, fillzero, C.byref(n), None)
    torch.cuda.synchronize()
    return rc, int(n.value), out[:cap]


def _existing(pkg, x, cs, dist):
    c = pkg.GPUCellList(tuple(x), cs, dist)
    return c.neighborlistview().clone()


def test_noalloc_pairs_match_existing_entry_point_twice(gpu_pkg):
    """Two calls in a row (2-D, then 3-D with different sizes, so the second
    call reuses an arena holding the first call's data) give the same list,
    in the same order, as gcl_create + gcl_emit_pairs; integer output, so the
    comparison is exact."""
    L = gpu_pkg.load_library()
    cases = [(gpu_pkg.workloads.uniform_points(60000, 2, seed=101), (0.02, 0.02), 0.02),
             (gpu_pkg.workloads.uniform_points(40000, 3, seed=202), (0.06, 0.06, 0.06), 0.06)]
    for x, cs, dist in cases:
        want = _existing(gpu_pkg, x, cs, dist)
        cap = int(want.shape[0]) + 11
        rc, n, got = _noalloc(L, x, cs, dist, cap)
        assert rc == 0, L.gcsph_last_error()
        assert n == want.shape[0]
        assert torch.equal(got[:n], want)
        assert int((got[n:] != 0).sum()) == 0          # zero tail (fillzero)


def test_noalloc_capacity_and_limits(gpu_pkg):
    L = gpu_pkg.load_library()
    x = gpu_pkg.workloads.uniform_points(5000, 2, seed=7)
    want = _existing(gpu_pkg, x, (0.05, 0.05), 0.05)
    rc, n, got = _noalloc(L, x, (0.05, 0.05), 0.05, 100)
    assert rc == 2 and n == want.shape[0]              # GCSPH_ECAPACITY, full count reported
    assert torch.equal(got, want[:100])
    # beyond the static scratch: rejected before any device work
    big = np.zeros((2, 262145))
    big[0] = np.linspace(0, 1, 262145)
    rc, n, _ = _noalloc(L, big, (0.1, 0.1), 0.1, 1)
    assert rc == 1 and b"static scratch" in L.gcsph_last_error()
    many_cells = gpu_pkg.workloads.uniform_points(1000, 2, seed=8)
    rc, n, _ = _noalloc(L, many_cells, (0.0005, 0.0005), 0.0005, 1)
    assert rc == 1 and b"cells" in L.gcsph_last_error()


def test_noalloc_near_its_limits(gpu_pkg):
    """262,144 uniform 2-D points (the point limit) on a 1001 x 1001 grid
    (cellsize = dist = 0.001, near the cell limit): both scans take the
    multi-tile path and the whole arena layout is in use.  Same list, in the
    same order, as gcl_create + gcl_emit_pairs, twice in a row."""
    L = gpu_pkg.load_library()
    N = 262144
    x = gpu_pkg.workloads.uniform_points(N, 2, seed=404)
    cs, dist = (0.001, 0.001), 0.001
    want = _existing(gpu_pkg, x, cs, dist)
    assert want.shape[0] > 50000
    for _ in range(2):
        rc, n, got = _noalloc(L, x, cs, dist, int(want.shape[0]))
        assert rc == 0, L.gcsph_last_error()
        assert n == want.shape[0] and torch.equal(got, want)


def test_noalloc_refuses_nan_coordinates(gpu_pkg):
    """Julia's minimum over a coordinate holding NaN is NaN and the
    constructor's ceil(Int, NaN) throws: the set has no cell grid.  The call
    says so instead of binning around the NaN."""
    L = gpu_pkg.load_library()
    x = gpu_pkg.workloads.uniform_points(1000, 3, seed=9)
    x[2, 17] = np.nan
    rc, n, _ = _noalloc(L, x, (0.1,) * 3, 0.1, 10)
    assert rc == 1 and b"NaN" in L.gcsph_last_error()


_FULL_DEVICE_SCRIPT = r"""
import ctypes as C, json, os, sys
import numpy as np
sys.path.insert(0, os.environ["GCSPH_ROOT"])
import torch
import __graft_entry__ as ge
from oracle import oracle as orc
g = ge.load_package()
L = g.load_library()
torch.cuda.set_device(0)
D, N, dist = 2, 50000, 0.01
x = g.workloads.uniform_points(N, D, seed=303)
cs_, off, cell = orc.grid(x, (dist, dist), dist)
pcell, _ = orc.cellmap(x, cs_, off, cell)
want, nwant = orc.neib_search(x, pcell, cell, dist)
xs = [torch.from_numpy(np.ascontiguousarray(x[d])).cuda() for d in range(D)]
ptrs = (C.c_void_p * 3)(*[t.data_ptr() for t in xs])
out = torch.zeros((nwant + 5, 2), dtype=torch.int32, device="cuda")
torch.cuda.synchronize()
rc0 = L.gcl_pairs_noalloc_init()
free0, _ = torch.cuda.mem_get_info()
hog = torch.empty(free0 - (16 << 20), dtype=torch.uint8, device="cuda")
free1, _ = torch.cuda.mem_get_info()
res = []
for _ in range(2):
    n = C.c_int64()
    rc = L.gcl_pairs_noalloc(D, N, C.cast(ptrs, C.POINTER(C.c_void_p)), (C.c_double * 3)(dist, dist, 0.0), dist,
                             None, None, C.c_void_p(out.data_ptr()), nwant + 5, 1, C.byref(n), None)
    got = out.cpu().numpy()
    same = bool(n.value == nwant and np.array_equal(orc.pair_set(got[:nwant]), orc.pair_set(want))
                and not got[nwant:].any())
    res.append({"rc": int(rc), "n": int(n.value), "same": same, "err": L.gcsph_last_error().decode()})
print(json.dumps({"init": int(rc0), "free_after_fill": int(free1), "calls": res}))
"""


def test_noalloc_after_the_device_is_full(gpu_pkg):
    """A fresh process loads the library, calls gcl_pairs_noalloc_init, then
    lets its own pool take all but 16 MiB of the device's free memory -- less
    than the static array itself, which CUDA reserves when it loads the
    library's code on the device (lazily, at the first use).  Both calls that
    follow still succeed and return the oracle's pair set and count."""
    env = dict(os.environ, GCSPH_ROOT=ROOT, CUDA_MODULE_LOADING="LAZY")
    r = subprocess.run([sys.executable, "-c", _FULL_DEVICE_SCRIPT], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["init"] == 0
    assert out["free_after_fill"] < 24 << 20
    for c in out["calls"]:
        assert c["rc"] == 0 and c["same"], c
