"""GPU parity of the cell list: the pair set from libgcsph.so must equal the
oracle's / the golden fixture's bit for bit (compared as sorted sets)."""
import ctypes as C
import math
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _set(orc, pairs):
    return orc.pair_set(pairs.cpu().numpy() if torch.is_tensor(pairs) else pairs)


def _oracle_pairs(orc, x, cs, dist, MIN=None, MAX=None):
    c, off, cell = orc.grid(x, cs, dist, MIN, MAX)
    pcell, cpn = orc.cellmap(x, c, off, cell)
    pairs, n = orc.neib_search(x, pcell, cell, dist)
    return pairs, n, (c, off, cell, pcell, cpn)


def _assert_maxpairs_and_capacity(c, orc, x, cs, dist, MIN=None, MAX=None):
    """c.maxpairs() equals the oracle's мaxpairs over the oracle's cellpnum
    (src/gpukernels_cls.jl:109-286), and the pair array's length is the
    constructor's policy applied to it (src/celllist.jl:69-86): capacity
    мaxpairs, shrunk to ceil(pairsn / 0.8) when less than 80% full."""
    D = len(cs)
    cs_, off, cell = orc.grid(x, cs, dist, MIN, MAX)
    _, cpn = orc.cellmap(x, cs_, off, cell)
    mp = orc.maxpairs(D, cpn, cell)
    assert c.maxpairs() == mp
    assert mp >= c.pairsn
    want_cap = math.ceil(c.pairsn / 0.8) if c.pairsn < mp * 0.8 else mp
    assert c.neighborlist().shape[0] == want_cap


def _golden_hash(pairs):
    import importlib.util
    spec = importlib.util.spec_from_file_location("mg", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.pair_hash(pairs)


@pytest.mark.parametrize("tag", ["H", "1p1H"])
def test_fixture_dp002_pairs_match_golden(gpu_pkg, orc, tag):
    z = np.load(os.path.join(GOLDEN, "dambreak2d_dp002.npz"))
    dist = float(z[f"pairs_{tag}_dist"])
    c = gpu_pkg.GPUCellList(tuple(z["x"]), (dist, dist), dist)
    assert c.pairsn == int(z[f"pairs_{tag}_n"])
    ps = _set(orc, c.neighborlistview())
    assert [int(v) for v in _golden_hash(ps)] == [int(v) for v in z[f"pairs_{tag}_hash"]]
    # README.md:51 identity, zero tail, (min,max) order
    full = c.neighborlist().cpu().numpy()
    assert int((full[:, 0] != 0).sum()) == c.pairsn
    v = full[: c.pairsn]
    assert (v[:, 0] < v[:, 1]).all() and v.min() >= 1 and v.max() <= c.n
    # мaxpairs (src/gpukernels_cls.jl:109-286) against the oracle's count of
    # the same cells, and the constructor's capacity policy built on it
    # (src/celllist.jl:69-86): the list length follows from that count alone
    _assert_maxpairs_and_capacity(c, orc, z["x"], (dist, dist), dist)


def test_fixture_dp004_full_set(gpu_pkg, orc):
    z = np.load(os.path.join(GOLDEN, "dambreak2d_dp004.npz"))
    dist = float(z["pairs_H_dist"])
    c = gpu_pkg.GPUCellList(tuple(z["x"]), (dist, dist), dist)
    assert np.array_equal(_set(orc, c.neighborlistview()), orc.pair_set(z["pairs_H"]))
    _assert_maxpairs_and_capacity(c, orc, z["x"], (dist, dist), dist)


def test_fixture_3d_boundary_hash(gpu_pkg, orc):
    z = np.load(os.path.join(GOLDEN, "dambreak3d_boundary.npz"))
    dist = float(z["pairs_dist"])
    c = gpu_pkg.GPUCellList(tuple(z["x"]), (dist,) * 3, dist)
    assert c.pairsn == int(z["pairs_n"])
    assert [int(v) for v in _golden_hash(_set(orc, c.neighborlistview()))] == [int(v) for v in z["pairs_hash"]]


@pytest.mark.parametrize("D,N,dist,seed", [(2, 20000, 0.016, 1), (3, 30000, 0.03, 2), (2, 3000, 0.3, 3),
                                           (3, 2000, 0.4, 4), (2, 1, 0.1, 5), (3, 2, 0.5, 6)])
def test_random_sets_match_oracle(gpu_pkg, orc, D, N, dist, seed):
    x = np.random.default_rng(seed).random((D, N))
    c = gpu_pkg.GPUCellList(tuple(x), (dist,) * D, dist)
    pairs, n, (cs, off, cell, pcell, cpn) = _oracle_pairs(orc, x, (dist,) * D, dist)
    assert c.pairsn == n
    assert np.array_equal(_set(orc, c.neighborlistview()), orc.pair_set(pairs))
    assert c.grid == tuple(int(v) for v in cell)
    assert np.allclose(c.offset, off, rtol=0, atol=0)
    assert np.array_equal(c.cellpnum.cpu().numpy(), cpn)
    assert c.maxpairs() == orc.maxpairs(D, cpn, cell)
    _assert_maxpairs_and_capacity(c, orc, x, (dist,) * D, dist)


def test_adversarial_points(gpu_pkg, orc):
    dist = 0.25
    pts = [(0.0, 0.0), (0.25, 0.0), (0.5, 0.5), (0.5, 0.5), (0.75, 0.0), (0.75, 0.2499999), (1.0, 1.0),
           (1.0, 0.75), (3.0, 3.0), (3.1, 3.05), (2.0, 0.0)]
    x = np.array(pts, dtype=np.float64).T.copy()
    c = gpu_pkg.GPUCellList(tuple(x), (dist, dist), dist)
    pairs, n, _ = _oracle_pairs(orc, x, (dist, dist), dist)
    got = {tuple(p) for p in _set(orc, c.neighborlistview()).tolist()}
    assert got == {tuple(p) for p in orc.pair_set(pairs).tolist()}
    assert (1, 2) not in got and (3, 4) in got


def test_clamped_cells_with_given_box(gpu_pkg, orc):
    x = np.random.default_rng(11).uniform(-0.5, 1.5, (3, 3000))
    dist = 0.1
    c = gpu_pkg.GPUCellList(tuple(x), (dist,) * 3, dist, MIN=(0, 0, 0), MAX=(1, 1, 1))
    pairs, n, _ = _oracle_pairs(orc, x, (dist,) * 3, dist, MIN=(0, 0, 0), MAX=(1, 1, 1))
    assert c.pairsn == n
    assert np.array_equal(_set(orc, c.neighborlistview()), orc.pair_set(pairs))
    _assert_maxpairs_and_capacity(c, orc, x, (dist,) * 3, dist, MIN=(0, 0, 0), MAX=(1, 1, 1))


def test_single_overfull_cell(gpu_pkg, orc):
    x = np.random.default_rng(12).uniform(0, 0.01, (2, 700))
    c = gpu_pkg.GPUCellList(tuple(x), (1.0, 1.0), 1.0)
    assert c.pairsn == 700 * 699 // 2
    assert int(c.cellpnum.max().item()) == 700


def test_update_and_partialupdate_follow_reference_semantics(gpu_pkg, orc):
    """update! re-bins moved points; partialupdate! keeps the stale cells
    (src/celllist.jl:95-145).  Both compared with the oracle's own sequence."""
    rng = np.random.default_rng(21)
    D, N, dist = 2, 20000, 0.016
    x = rng.random((D, N))
    c = gpu_pkg.GPUCellList(tuple(x), (dist, dist), dist)
    p = orc.default_params(0.01, 0.01, 0.016, 1000, 0.1, 1e-5, 0.01, 10, 7, 0.1, 0.2, dist)
    o = orc.OracleSystem(x, (dist, dist), dist, np.full(N, 1000.0), np.full(N, 2, np.int32), p)
    x2 = x + rng.uniform(-0.6, 0.6, x.shape) * dist
    for d in range(D):
        c.points[d].copy_(torch.from_numpy(x2[d]))
    o.set_x(x2)
    c.partialupdate()
    o.partialupdate()
    assert c.pairsn == o.pairsn
    assert np.array_equal(_set(orc, c.neighborlistview()), orc.pair_set(o.pairs()[: o.pairsn]))
    c.update()
    o.update()
    assert c.pairsn == o.pairsn
    assert np.array_equal(_set(orc, c.neighborlistview()), orc.pair_set(o.pairs()[: o.pairsn]))
    full = c.neighborlist().cpu().numpy()
    assert int((full[:, 0] != 0).sum()) == c.pairsn   # README.md:58


def test_emit_reports_capacity_overflow(gpu_pkg):
    from importlib import import_module
    L = gpu_pkg.load_library()
    lib_mod = import_module(gpu_pkg.__name__ + "._lib")
    x = np.random.default_rng(4).random((2, 5000))
    c = gpu_pkg.GPUCellList(tuple(x), (0.05, 0.05), 0.05)
    small = torch.zeros((10, 2), dtype=torch.int32, device="cuda")
    n = C.c_int64()
    rc = L.gcl_emit_pairs(c._h, C.c_void_p(small.data_ptr()), 10, 1, C.byref(n))
    assert rc == lib_mod.GCSPH_ECAPACITY and n.value == c.pairsn
    # the first 10 pairs are the first 10 of the full list
    assert torch.equal(small, c.neighborlistview()[:10])


def test_emit_into_a_buffer_not_8_byte_aligned(gpu_pkg):
    """A caller's pair buffer that starts 4 bytes into an allocation: the
    emit stores 4-byte words there instead of pair-wide ones; the contents
    equal those of the aligned emit, capacity cut included."""
    L = gpu_pkg.load_library()
    x = np.random.default_rng(5).random((2, 20000))
    c = gpu_pkg.GPUCellList(tuple(x), (0.02, 0.02), 0.02)
    want = c.neighborlistview().clone()
    n = C.c_int64()
    for cap in (c.pairsn, c.pairsn // 3):
        raw = torch.full((2 * c.pairsn + 2,), -7, dtype=torch.int32, device="cuda")
        ptr = raw.data_ptr() + 4
        assert ptr % 8 == 4
        rc = L.gcl_emit_pairs(c._h, C.c_void_p(ptr), cap, 0, C.byref(n))
        assert n.value == c.pairsn and (rc == 0) == (cap == c.pairsn)
        got = raw[1:1 + 2 * cap].view(cap, 2)
        assert torch.equal(got, want[:cap])
        assert int(raw[0]) == -7 and int(raw[1 + 2 * cap]) == -7  # nothing written outside


@pytest.mark.parametrize("D,N,dist", [(2, 200_000, 0.016), (3, 4_000_000, 0.008)])
def test_full_size_pair_sets(gpu_pkg, orc, D, N, dist):
    """The cell-list configuration at full size: 200k 2-D / 4M 3-D uniform
    points, pair sets and мaxpairs compared with the oracle, then a jittered
    partialupdate! compared by count and set."""
    x = gpu_pkg.workloads.uniform_points(N, D)
    c = gpu_pkg.GPUCellList(tuple(x), (dist,) * D, dist)
    pairs, n, (_, _, cell, pcell, cpn) = _oracle_pairs(orc, x, (dist,) * D, dist)
    assert c.pairsn == n
    assert c.maxpairs() == orc.maxpairs(D, cpn, cell)

    def same_set(got, want):
        got = got.astype(np.int64)
        assert (got[:, 0] < got[:, 1]).all()
        want = want.astype(np.int64)
        kg = np.sort(got[:, 0] * (1 << 32) + got[:, 1])
        kw = np.sort(want[:, 0] * (1 << 32) + want[:, 1])
        assert np.array_equal(kg, kw)
        assert np.unique(kg).size == kg.size

    same_set(c.neighborlistview().cpu().numpy(), pairs)
    del pairs
    # partialupdate! (src/celllist.jl:141-145): every point jittered by
    # U(-0.1, 0.1)·dist per coordinate, the pair search re-run with the cell
    # membership of the build above (stale cells) and the new coordinates;
    # the oracle does the same with its own stale pcell
    rng = np.random.default_rng(7)
    xj = np.ascontiguousarray(x + rng.uniform(-0.1, 0.1, x.shape) * dist)
    for d in range(D):
        c.points[d].copy_(torch.from_numpy(xj[d]))
    c.partialupdate()
    pj, nj = orc.neib_search(xj, pcell, cell, dist)
    assert c.pairsn == nj
    same_set(c.neighborlistview().cpu().numpy(), pj)


@pytest.mark.parametrize("D", [2, 3])
def test_tiny_and_degenerate_sets(gpu_pkg, orc, D):
    """One point (no pairs); two coincident points (r² = 0 < dist²: one pair);
    two points exactly dist apart (the reference's test is strict: no pair);
    every case against the oracle.  An empty set is refused, as the
    reference's bounding box of no points is an error, and so is a set with
    a NaN coordinate."""
    dist = 0.1
    cases = {
        "one": np.full((D, 1), 0.5),
        "coincident": np.full((D, 2), 0.5),
        "exactly_dist": np.zeros((D, 2)),
        "far": np.array([[0.0, 1.0]] + [[0.0, 0.0]] * (D - 1)),
    }
    cases["exactly_dist"][0, 1] = dist
    want = {"one": 0, "coincident": 1, "exactly_dist": 0, "far": 0}
    for name, x in cases.items():
        x = np.ascontiguousarray(x, dtype=np.float64)
        c = gpu_pkg.GPUCellList(tuple(x), (dist,) * D, dist)
        pairs, n, _ = _oracle_pairs(orc, x, (dist,) * D, dist)
        assert c.pairsn == n == want[name], (name, c.pairsn, n)
        got = _set(orc, c.neighborlistview())
        assert np.array_equal(got, orc.pair_set(pairs)), name
        c.update()
        assert c.pairsn == want[name], name
    with pytest.raises(RuntimeError):
        gpu_pkg.GPUCellList(tuple(np.zeros((D, 0))), (dist,) * D, dist)
    # a NaN coordinate: Julia's minimum is NaN and ceil(Int, NaN) throws in
    # the constructor (src/celllist.jl:41-46); refused here as well
    bad = np.full((D, 4), 0.5)
    bad[D - 1, 2] = np.nan
    with pytest.raises(RuntimeError, match="NaN"):
        gpu_pkg.GPUCellList(tuple(bad), (dist,) * D, dist)


def test_one_crowded_cell(gpu_pkg):
    """10^5 points in one cell (cellsize 1 over the unit square, dist 0.002):
    sets of this size take the stable radix sort, whose cost has no term in
    the square of a cell's population, and update! (binning + pair search)
    completes in under 50 ms after a warm-up.  The pair set equals the
    reference's test r² < dist² (every pair of this grid is a candidate),
    evaluated here from scipy cKDTree candidates."""
    import time
    from scipy.spatial import cKDTree
    N, dist = 100_000, 0.002
    x = gpu_pkg.workloads.uniform_points(N, 2, seed=31)
    c = gpu_pkg.GPUCellList(tuple(x), (1.0, 1.0), dist)
    assert int(c.cellpnum.max().item()) > N // 4
    c.update()
    ts = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c.update()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    print(f"\n[crowded cell] update! of {N} points in {len(c.grid)}-D grid {c.grid}: {min(ts) * 1e3:.2f} ms")
    assert min(ts) < 0.050
    cand = cKDTree(x.T).query_pairs(dist * (1 + 1e-7), output_type="ndarray")
    i, j = cand[:, 0], cand[:, 1]
    d0 = x[0, i] - x[0, j]
    d1 = x[1, i] - x[1, j]
    keep = (d0 * d0 + d1 * d1) < dist * dist
    want = np.sort((np.minimum(i, j)[keep] + 1) * (1 << 32) + np.maximum(i, j)[keep] + 1)
    got = c.neighborlistview().cpu().numpy().astype(np.int64)
    assert c.pairsn == want.size
    assert np.array_equal(np.sort(got[:, 0] * (1 << 32) + got[:, 1]), want)


@pytest.mark.parametrize("D,N", [(2, 200_000), (3, 300_000)])
def test_sort_choices_same_pair_list(gpu_pkg, D, N):
    """The three in-cell orderings of a large set (by the most crowded cell,
    the counting sort's rank, the stable radix sort) give the same pair list
    in the same order, for update! and partialupdate! alike."""
    x = gpu_pkg.workloads.uniform_points(N, D, seed=7 + D)
    dist = 0.006 if D == 2 else 0.02
    lists = []
    for mode in (0, 1, 2):
        c = gpu_pkg.GPUCellList(tuple(x), (dist,) * D, dist)
        c.set_sort(mode)
        c.update()
        c.partialupdate()
        lists.append(c.neighborlistview().clone())
        c.close()
    assert lists[0].shape[0] > N
    assert torch.equal(lists[0], lists[1]) and torch.equal(lists[1], lists[2])


def test_set_sort_rejects_unknown_mode(gpu_pkg):
    x = gpu_pkg.workloads.uniform_points(1000, 2, seed=3)
    c = gpu_pkg.GPUCellList(tuple(x), (0.05, 0.05), 0.05)
    with pytest.raises(RuntimeError):
        c.set_sort(3)
    c.close()
