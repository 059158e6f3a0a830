"""Generate the committed golden fixtures from the reference's test inputs.

Run where a checkout of the reference exists (read-only), with its path:
    python tests/golden/make_golden.py <path of the reference checkout>
Nothing at test time reads the reference; the .npz files written here are
the fixtures.

What is pinned:
  * inputs: the reference's own particle CSVs (test/input/*.csv) converted
    to float64/int32 arrays, exactly as loadparticles / the README demo read
    them (columns Points:0, Points:2 [, Points:1], Rhop, ptype).
  * the pair set of GPUCellList(points, (H,H), dist) for those inputs,
    computed HERE by an implementation independent of both the oracle and the
    CUDA library: scipy cKDTree candidates within dist*(1+1e-7), then the
    reference's exact test -- clamped cells (src/gpukernels_cls.jl:29-60) within
    Chebyshev distance 1 and r^2 = (xi-xj)^2 + (yi-yj)^2 [+ (zi-zj)^2] < dist^2
    evaluated left to right in IEEE float64 (src/gpukernels_cls.jl:326,390).
    Small sets are stored in full, large ones as (count, two 64-bit hashes).
The reference itself (Julia + CUDA.jl, GPU-only) cannot run here, so no
field values beyond the pair set are pinned.
"""
from __future__ import annotations

import csv
import math
import os
import sys

import numpy as np
from scipy.spatial import cKDTree

HERE = os.path.dirname(os.path.abspath(__file__))
SQRT_EPS = 1.4901161193847656e-08


def read_csv(path, cols):
    with open(path, newline="") as f:
        rows = list(csv.DictReader(f))
    return rows, [np.array([float(r[c]) for r in rows]) for c in cols]


def grid(x, cs, dist):
    D = x.shape[0]
    cs = np.array([max(c, dist) for c in cs])
    mn = x.min(axis=1)
    mx = x.max(axis=1)
    mn = mn - np.abs((mn + SQRT_EPS) * SQRT_EPS)
    cell = np.ceil((mx - mn) / cs).astype(np.int64)
    return cs, mn, cell


def cellmap(x, cs, off, cell):
    hinv = 1.0 / cs
    p = (x - off[:, None]) * hinv[:, None]
    c = np.minimum(np.maximum(p, 1.0), cell[:, None].astype(np.float64))
    return np.ceil(c).astype(np.int64)


def pair_set(x, cs_in, dist):
    D, N = x.shape
    cs, off, cell = grid(x, cs_in, dist)
    pc = cellmap(x, cs, off, cell)
    tree = cKDTree(x.T)
    cand = tree.query_pairs(dist * (1 + 1e-7), output_type="ndarray").astype(np.int64)
    i, j = cand[:, 0], cand[:, 1]
    r2 = (x[0, i] - x[0, j]) * (x[0, i] - x[0, j]) + (x[1, i] - x[1, j]) * (x[1, i] - x[1, j])
    if D == 3:
        r2 = r2 + (x[2, i] - x[2, j]) * (x[2, i] - x[2, j])
    near = np.all(np.abs(pc[:, i] - pc[:, j]) <= 1, axis=0)
    keep = near & (r2 < dist * dist)
    a = np.minimum(i[keep], j[keep]) + 1
    b = np.maximum(i[keep], j[keep]) + 1
    order = np.lexsort((b, a))
    return np.stack([a[order], b[order]], axis=1).astype(np.int32)


def pair_hash(pairs):
    """Order-independent hashes of a pair set (sum and xor of a 64-bit mix)."""
    a = pairs[:, 0].astype(np.uint64)
    b = pairs[:, 1].astype(np.uint64)
    with np.errstate(over="ignore"):
        k = a * np.uint64(0x9E3779B97F4A7C15) + b * np.uint64(0xC2B2AE3D27D4EB4F) + np.uint64(0x165667B19E3779F9)
        k ^= k >> np.uint64(29)
        k *= np.uint64(0xBF58476D1CE4E5B9)
        k ^= k >> np.uint64(32)
        s = np.sum(k, dtype=np.uint64)
    x = np.bitwise_xor.reduce(k) if k.size else np.uint64(0)
    return int(s), int(x)


def main(ref):
    inp = os.path.join(ref, "test", "input")
    out = {}
    # 2-D Dp0.02 with ptype column (README demo / test/runtests.jl input)
    _, (fx, fy, frho, fpt) = read_csv(os.path.join(inp, "FluidPoints_Dp0.02.csv"),
                                     ["Points:0", "Points:2", "Rhop", "ptype"])
    _, (bx, by, brho, bpt) = read_csv(os.path.join(inp, "BoundaryPoints_Dp0.02.csv"),
                                     ["Points:0", "Points:2", "Rhop", "ptype"])
    x = np.stack([np.concatenate([fx, bx]), np.concatenate([fy, by])])
    rho = np.concatenate([frho, brho])
    pt = np.concatenate([fpt, bpt]).astype(np.int32)
    dx = 0.02
    h = 1.2 * math.sqrt(2) * dx
    H = 2 * h
    res = {"x": x, "rho": rho, "ptype": pt, "dx": np.float64(dx)}
    for tag, dist in (("H", H), ("1p1H", 1.1 * H)):
        ps = pair_set(x, (dist, dist), dist)
        s, xr = pair_hash(ps)
        res[f"pairs_{tag}_n"] = np.int64(len(ps))
        res[f"pairs_{tag}_hash"] = np.array([s, xr], dtype=np.uint64)
        res[f"pairs_{tag}_dist"] = np.float64(dist)
        out[f"dp002 {tag}"] = len(ps)
    np.savez_compressed(os.path.join(HERE, "dambreak2d_dp002.npz"), **res)
    # 2-D Dp0.04 (no ptype column: Type 3 = fluid -> 2, else boundary -> 0), full pair set
    _, (fx, fy, frho, ft) = read_csv(os.path.join(inp, "FluidPoints_Dp0.04.csv"),
                                     ["Points:0", "Points:2", "Rhop", "Type"])
    _, (bx, by, brho, bt) = read_csv(os.path.join(inp, "BoundaryPoints_Dp0.04.csv"),
                                     ["Points:0", "Points:2", "Rhop", "Type"])
    x = np.stack([np.concatenate([fx, bx]), np.concatenate([fy, by])])
    typ = np.concatenate([ft, bt])
    pt = np.where(typ == 3, 2, 0).astype(np.int32)
    rho = np.concatenate([frho, brho])
    dx = 0.04
    h = 1.2 * math.sqrt(2) * dx
    H = 2 * h
    ps = pair_set(x, (H, H), H)
    np.savez_compressed(os.path.join(HERE, "dambreak2d_dp004.npz"), x=x, rho=rho, ptype=pt, dx=np.float64(dx),
                        pairs_H=ps, pairs_H_dist=np.float64(H))
    out["dp004 H"] = len(ps)
    # 3-D boundary fixture (examples/timesolve3d.jl:13 axis map: Points:0, Points:2, Points:1)
    _, (x0, x2, x1) = read_csv(os.path.join(inp, "3D_DamBreak_Boundary.csv"), ["Points:0", "Points:2", "Points:1"])
    x = np.stack([x0, x2, x1])
    dx = 0.0085
    h = math.sqrt(3 * dx ** 2)
    H = 2 * h
    dist = 1.1 * H
    ps = pair_set(x, (dist, dist, dist), dist)
    s, xr = pair_hash(ps)
    np.savez_compressed(os.path.join(HERE, "dambreak3d_boundary.npz"), x=x, dx=np.float64(dx),
                        pairs_n=np.int64(len(ps)), pairs_hash=np.array([s, xr], dtype=np.uint64),
                        pairs_dist=np.float64(dist))
    out["3d boundary 1.1H"] = len(ps)
    for k, v in out.items():
        print(f"{k}: {v} pairs")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
