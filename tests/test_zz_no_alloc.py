"""gcl_pairs_noalloc: the pair list in one call that allocates no device memory.

It exists for callers that may not allocate device memory while they run (a
process whose own pool already holds the GPU, a plugin host that forbids it,
a time-critical loop that cannot absorb cudaMalloc's implicit synchronisation).
This file is collected last so that a failure here stops a `-x` run only
after every other test has run; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

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
