"""GPUCellList -- host-side mirror of src/celllist.jl over libgcsph.so.

Same constructor arguments, fields, capacity policy and error behaviour as
the Julia struct; the binning and the pair search run in the CUDA library.
Python names drop Julia's `!`: update! -> update, partialupdate! ->
partialupdate.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings

import torch

from . import _lib


def _as_points(points):
    """CuArray{T}.(points): a CUDA float64 copy of each coordinate array."""
    pts = []
    for p in points:
        t = torch.as_tensor(p)
        t = t.to(device="cuda", dtype=torch.float64).contiguous().clone()
        pts.append(t)
    return tuple(pts)


class GPUCellList:
    """GPUCellList(points, cellsize, dist; MIN, MAX, mppcell, mpairs) -- src/celllist.jl:22-88.

    points: tuple of D (2 or 3) equal-length coordinate arrays.
    Fields: n, dist, cs, offset, grid, points, cellpnum (Int32, column-major
    over grid, flattened), pairs (cap x 2 int32, 1-based (min,max), zero tail),
    pairsn.  The dense `celllist` and `pcell` arrays of the reference are not
    kept: cell membership lives in the library's sorted order.
    """

    def __init__(self, points, cellsize, dist, MIN=None, MAX=None, mppcell=0, mpairs=0, stream=None):
        L = _lib.load()
        pl = [len(p) for p in points]
        if not all(x == pl[0] for x in pl):
            raise ValueError("length of points not equal")
        D = len(points)
        if D < 2 or D > 3:
            raise ValueError("wrong dimention")
        dist = float(dist)
        cs = [float(c) for c in cellsize]
        for i in range(D):
            if cs[i] < dist:
                warnings.warn(f"Cell size (dim {i + 1}) < dist, cell size set equal dist")
                cs[i] = dist
        self.points = _as_points(points)
        self.n = int(pl[0])
        self.dim = D
        self.dist = dist
        self._stream = stream
        mn = None if MIN is None else (C.c_double * 3)(*[float(v) for v in MIN])
        mx = None if MAX is None else (C.c_double * 3)(*[float(v) for v in MAX])
        h = C.c_void_p()
        _lib.check(L.gcl_create(D, self.n, _lib.ptrs(self.points), (C.c_double * 3)(*cs), dist,
                                mn, mx, C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h
        csv = (C.c_double * 3)(); off = (C.c_double * 3)(); cell = (C.c_int64 * 3)()
        _lib.check(L.gcl_grid(h, csv, off, cell))
        self.cs = tuple(csv[i] for i in range(D))
        self.offset = tuple(off[i] for i in range(D))
        self.grid = tuple(int(cell[i]) for i in range(D))
        self._refresh_cellpnum()
        # mppcell is reported for API parity (the dense cell list is not built)
        self.mppcell = max(int(mppcell), int(math.ceil(int(self.cellpnum.max().item()) * 1.05 + 1)))
        if mpairs == 0:
            mp = C.c_int64()
            _lib.check(L.gcl_maxpairs(h, C.byref(mp)))
            mpairs = int(mp.value)
        mpairs = int(mpairs)
        # celllist.jl:73-86: capacity mpairs, shrink to ceil(total/0.8) if < 80% full
        self.pairs = torch.zeros((max(mpairs, 0), 2), dtype=torch.int32, device="cuda")
        total = self._emit(fillzero=True, allow_overflow=True)
        if total > mpairs:
            warnings.warn("List of pairs not full, call `update!(c::GPUCellList)` to extend pair list!")
        if total < mpairs * 0.8:
            new_pairn = int(math.ceil(total / 0.8))
            self.pairs = self.pairs[:new_pairn].clone()
        self.pairsn = total

    # ------------------------------------------------------------------ internals
    def _refresh_cellpnum(self):
        ncell = 1
        for g in self.grid:
            ncell *= g
        self.cellpnum = torch.empty(ncell, dtype=torch.int32, device="cuda")
        _lib.check(_lib.load().gcl_cellpnum(self._h, _lib.dptr(self.cellpnum)))

    def _emit(self, fillzero=True, allow_overflow=False) -> int:
        n = C.c_int64()
        cap = int(self.pairs.shape[0])
        rc = _lib.load().gcl_emit_pairs(self._h, _lib.dptr(self.pairs) if cap else None, cap,
                                         int(bool(fillzero)), C.byref(n))
        _lib.check(rc, allow=(_lib.GCSPH_ECAPACITY,) if allow_overflow else ())
        return int(n.value)

    def _apply_update_policy(self, prev_pairsn: int, total: int, fillzero: bool):
        """Capacity policy of update!, src/celllist.jl:117-133."""
        cap = int(self.pairs.shape[0])
        realloc = False
        if prev_pairsn > cap or prev_pairsn < cap * 0.6:
            cap = int(math.ceil(prev_pairsn / 0.8))
            realloc = True
        if total > cap:
            cap = int(math.ceil(total / 0.8))
            realloc = True
        if realloc:
            self.pairs = torch.zeros((cap, 2), dtype=torch.int32, device="cuda")
        self._emit(fillzero=fillzero or realloc)
        self.pairsn = total

    # ------------------------------------------------------------------ API
    def update(self, fillzero: bool = True):
        """update!(c, fillzero) -- src/celllist.jl:95-134."""
        n = C.c_int64()
        _lib.check(_lib.load().gcl_update(self._h, C.byref(n)))
        self._refresh_cellpnum()
        self._apply_update_policy(self.pairsn, int(n.value), fillzero)

    def partialupdate(self, fillzero: bool = True):
        """partialupdate!(c, fillzero) -- src/celllist.jl:141-145 (no reallocation)."""
        n = C.c_int64()
        _lib.check(_lib.load().gcl_partialupdate(self._h, C.byref(n)))
        self._emit(fillzero=fillzero, allow_overflow=True)
        self.pairsn = int(n.value)

    def neighborlist(self):
        """neighborlist(c) -- src/celllist.jl:152-154: the whole pair array."""
        return self.pairs

    def neighborlistview(self):
        """neighborlistview(c) -- src/celllist.jl:161-163: pairs[1:pairsn]."""
        return self.pairs[: self.pairsn]

    def maxpairs(self) -> int:
        mp = C.c_int64()
        _lib.check(_lib.load().gcl_maxpairs(self._h, C.byref(mp)))
        return int(mp.value)

    def set_sort(self, mode: int):
        """The order inside a cell of the binning (no reference counterpart):
        0 = chosen by the most crowded cell (default), 1 = the counting sort's
        in-cell rank, 2 = the stable radix sort (sets above 65,536 points).
        The pair list and every result are the same for each choice."""
        _lib.check(_lib.load().gcl_set_sort(self._h, int(mode)))

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.load().gcl_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __repr__(self):
        g = "X".join(str(v) for v in self.grid)
        return (f"    Cell List (Dim: {self.dim})\n  Points number: {self.n} Type: Float64\n"
                f"  Pairs number: {self.pairsn}\n  Cell grid: {g}\n  Cutoff: {self.dist}")


def update(c: GPUCellList, fillzero: bool = True):
    c.update(fillzero)


def partialupdate(c: GPUCellList, fillzero: bool = True):
    c.partialupdate(fillzero)


def neighborlist(c: GPUCellList):
    return c.neighborlist()


def neighborlistview(c: GPUCellList):
    return c.neighborlistview()
