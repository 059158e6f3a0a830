"""Benchmark: particle-steps/s of the FP64 drop-in stepsolve! on one GB300.

Workload (default): 2-D dam break, plain FP64 single instance -- fluid column
1.0 x 2.0 m at dx = 0.02 (5,000 particles, ρ = 1000, v = 0) in a 4.0 x 3.0 m
tank with 3 lattice rows of fixed boundary particles (ptype 0), WendlandC2 2-D,
h = 1.2√2·dx, H = 2h, cellsize (H, H), dist = H (cell list rebuilt every
step), α = 0.01, g = 9.81, c₀ = 20√(2g), γ = 7, δ = 0.1, Δt = 1e-5.
One bench step = stepsolve!(prob, 15): 15 SPH time steps, one CSPM period.
Timed with CUDA events on the library's stream (the legacy default stream);
the L2 is flushed (256 MB write) between bench steps, outside the events.

--impl reference times the CPU restatement of the reference's algorithm (the
reference itself is Julia + CUDA.jl and cannot run here) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SUB = 15                    # SPH steps per bench step (one CSPM period)
WORKLOAD = "2-D dam break, plain FP64 single instance, dx=0.02, 1.0x2.0 m column in 4.0x3.0 m tank, 3 boundary rows"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-batched", action="store_true", help="skip the batched FP32 ensemble measurement")
    ap.add_argument("--batched-instances", type=int, default=256)
    ap.add_argument("--batched-steps", type=int, default=300, help="timed steps of the ensemble")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--serving-requests", type=int, default=40)
    ap.add_argument("--serving-horizon-scale", type=float, default=0.01)
    ap.add_argument("--serving-policy", default="shortest", choices=["shortest", "arrival"])
    ap.add_argument("--serving-caps", default="1500000,500000",
                    help="shortest-first: 2-D and 3-D particles in flight")
    ap.add_argument("--no-celllist", action="store_true", help="skip the cell-list update!/partialupdate! timing")
    ap.add_argument("--c3", action="store_true",
                    help="instead: 3-D dam break at scale, FP32 ensemble against the FP64 drop-in (one JSON line)")
    ap.add_argument("--c3-steps", type=int, default=500)
    ap.add_argument("--c3-dx", type=float, default=0.01)
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float) -> float:
    """The largest x over all ranks of the current process group (the slowest
    replica's time); x itself without one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_case(pkg):
    return pkg.workloads.dam_break_2d()


def algorithmic_bytes_per_stage(case, npairs):
    """Algorithmic HBM bytes of one pair-once pass A (FP64), the dominant
    kernel: N·(8D x + 8D v + 8 ρ + 8 P + 8 1/ρ + 4 ptype) of particle state
    read once, P·16 B of pair quads read, and per pair both sides' entry
    slots written: 2·(8 W + 8D ∇W + 8 ρ̇ + 8D a) B (stage 1; stage 2 writes
    no W/∇W).  P = pairs with k < m."""
    D, N = case.D, case.N
    return N * (16 * D + 28) + npairs * (16 + 2 * (16 + 16 * D))


def algorithmic_flops_stage1(case, x, v):
    """Algorithmic FP64 flops of one stage-1 pass A launch: every pair once,
    the reference's per-pair expressions counted as written (add, mul, cmp,
    div, sqrt = 1 each; the reference's own arithmetic has no FMA):
      sphW! + sph∇W! (every pair): 7D + 16
      ∂ρ∂tDDT! (both real): 7D + 1, and 34 per fluid side (powfancy7th 22 of it)
      ∂v∂t! (both real): 3D + 4
      ∂v∂t_av! (both real): 3D, and 5D + 10 more where Δv·Δx < 0
      fbmolforce! (one side real): 3D + 1, and 3D + 14 more where r < r₀ = 2dx
    The two data-dependent branches are counted for the pairs that take them
    in the state (x, v) given; the pairs are those with r <= dist in x (a
    pair exactly at dist, which the reference drops, changes the count by
    one pair's flops)."""
    import numpy as np
    from scipy.spatial import cKDTree
    D = case.D
    pt = np.asarray(case.ptype)
    pr = cKDTree(np.ascontiguousarray(x.T)).query_pairs(case.dist, output_type="ndarray")
    i, j = pr[:, 0], pr[:, 1]
    dxv = x[:, i] - x[:, j]
    dvv = v[:, i] - v[:, j]
    real = (pt[i] > 0) & (pt[j] > 0)
    mixed = (pt[i] > 0) != (pt[j] > 0)
    fluid_sides = (pt[i] > 1).astype(np.int64) + (pt[j] > 1)
    approach = real & ((dvv * dxv).sum(axis=0) < 0)
    inside = mixed & (np.sqrt((dxv * dxv).sum(axis=0)) < 2.0 * case.dx)
    flops = ((7 * D + 16) * len(i) + real.sum() * ((7 * D + 1) + (3 * D + 4) + 3 * D) +
             34 * fluid_sides[real].sum() + (5 * D + 10) * approach.sum() +
             (3 * D + 1) * mixed.sum() + (3 * D + 14) * inside.sum())
    return int(flops), {"pairs": int(len(i)), "real": int(real.sum()), "one_side_real": int(mixed.sum()),
                        "approaching": int(approach.sum()), "within_r0": int(inside.sum())}


# DRAM bytes (read + write) of one stage-1 pass A launch on this workload, from
# the ncu capture summarised in profiles/pairA_dambreak2d_c1_fp64.md
PAIRA_STAGE1_DRAM_BYTES = 2_100_992 + 512
PAIRA_STAGE1_FP64_PIPE = 0.777


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        import tempfile
        out = os.environ.get("GCSPH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out, f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
            # nvidia-smi's start-up (NVML initialisation) stalls CUDA calls of
            # this process for up to ~100 ms: the timed region starts only
            # once the sampler has written its first sample
            for _ in range(300):
                if os.path.getsize(self.path) > 0:
                    break
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1])); mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(case, seconds, threads):
    """The oracle (C restatement of the reference's pair loops) on host cores,
    a bounded sample of the same workload: whole bench steps until `seconds`."""
    from oracle import oracle as orc
    orc.set_threads(threads)
    p = orc.default_params(case.dx, case.h, case.H, case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma,
                           case.delta, case.CFL, case.dist)
    s = orc.OracleSystem(case.x, case.cellsize, case.dist, case.rho, case.ptype, p)
    s.stepsolve(1)
    n = 0
    t0 = time.perf_counter()
    while True:
        s.stepsolve(SUB)
        n += SUB
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return case.N * n / el, n, el


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__ as ge
    wl = ge.load_package().workloads  # importing the package needs no GPU
    from oracle import oracle as orc
    case = wl.dam_break_2d()
    threads = orc.max_threads()
    orc.set_threads(threads)
    p = orc.default_params(case.dx, case.h, case.H, case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma,
                           case.delta, case.CFL, case.dist)
    s = orc.OracleSystem(case.x, case.cellsize, case.dist, case.rho, case.ptype, p)
    for _ in range(args.warmup):
        s.stepsolve(SUB)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        s.stepsolve(SUB)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = case.N * SUB * args.steps / total
    out = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "impl": "reference",
           "config": {"workload": WORKLOAD, "particles": case.N, "sph_steps_per_bench_step": SUB},
           "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                            "sample": f"{args.steps} x stepsolve!(prob, {SUB}) on the full workload"},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / n) if n > 0 else float(np.linalg.norm(a - b))


def plain_fp64_rate(g, cases, steps=30):
    """particle-steps/s of the FP64 drop-in path (stepsolve!, captured calls)
    on each case alone, summed over the sample."""
    import torch
    tot_ps, tot_s = 0, 0.0
    for case in cases:
        system = g.GPUCellList(tuple(case.x), case.cellsize, case.dist)
        prob = g.SPHProblem(system, case.dx, case.h, case.H, g.WendlandC2(dim=case.D), case.rho, case.ptype,
                            case.rho0, case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL)
        prob.stepsolve(steps)  # sizes the buffers (first call runs per step)
        prob.stepsolve(steps)  # captures
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prob.stepsolve(steps)
        torch.cuda.synchronize()
        tot_s += time.perf_counter() - t0
        tot_ps += case.N * steps
        prob.close()
        del system
    return tot_ps / tot_s


def fp32_error_vs_fp64(g, case, alpha, delta, steps=100):
    """Relative L2 error of the FP32 ensemble against the FP64 drop-in path
    (itself bit-identical / within 1e-12 of the reference algorithm) after
    `steps` steps of one instance."""
    spec = g.spec_from_case(case, alpha=alpha, delta=delta)
    ens = g.Ensemble(case.D)
    slot = ens.add(spec)
    ens.step(steps)
    system = g.GPUCellList(tuple(case.x), case.cellsize, case.dist)
    prob = g.SPHProblem(system, case.dx, case.h, case.H, g.WendlandC2(dim=case.D), case.rho, case.ptype,
                        case.rho0, case.m0, case.dt, alpha, case.c0, case.gamma, delta, case.CFL)
    prob.stepsolve(steps)
    import torch
    x64 = torch.stack(system.points).cpu().numpy()
    out = {"rho": rel_l2(ens.get(slot, "rho"), prob.rho.cpu().numpy()),
           "rho_minus_rho0": rel_l2(ens.get(slot, "rho") - case.rho0, prob.rho.cpu().numpy() - case.rho0),
           "v": rel_l2(ens.get(slot, "v"), torch.stack(prob.v).cpu().numpy()),
           "displacement": rel_l2(ens.get(slot, "x") - case.x, x64 - case.x),
           "steps": steps, "particles": case.N}
    ens.close()
    prob.close()
    return out


def run_batched(g, args, plain_c1):
    """The batched-ensemble workload: 256 independent 2-D dam breaks
    (fluid-column counts log-uniform 2k-200k, aspect 0.5-4, dx 0.005-0.02,
    α 0.005-0.05, δ 0.05-0.2), FP32, all advanced together."""
    import torch
    wl = g.workloads.ensemble_2d(args.batched_instances)
    ens = g.Ensemble(2)
    t0 = time.perf_counter()
    slots = [ens.add(g.spec_from_case(case, alpha=al, delta=de)) for case, al, de in wl]
    t_admit = time.perf_counter() - t0
    tot = ens.totals()
    ens.step(30)  # tuning (block size, list lanes, list tiling: 24 steps) + warm-up
    ens.step(args.batched_steps)  # captures the graph of this many steps
    torch.cuda.synchronize()
    L = g.load_library()
    L.gcsph_timing_enable(0)
    builds0 = sum(ens.list_builds(s) for s in slots)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    ens.step(args.batched_steps)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    builds = sum(ens.list_builds(s) for s in slots) - builds0
    value = tot["particles"] * args.batched_steps / (ms / 1e3)
    # instrumented pass for the per-kernel split
    L.gcsph_timing_enable(1)
    L.gcsph_timing_reset()
    ens.step(20)
    import ctypes as C
    fam = {}
    for tid in range(L.gcsph_timing_count()):
        n_ = C.c_int64(); t_ = C.c_double()
        L.gcsph_timing_get(tid, C.byref(n_), C.byref(t_))
        if n_.value:
            fam[L.gcsph_timing_name(tid).decode()] = {"launches": int(n_.value), "total_ms": float(t_.value)}
    L.gcsph_timing_enable(0)
    tuning = ens.tuning()
    skin = ens.skin()
    ens.close()
    sizes = sorted(wl, key=lambda t: t[0].N)
    sample = [sizes[0][0], sizes[len(sizes) // 2][0], sizes[-1][0]]
    plain = plain_fp64_rate(g, sample)
    small = sizes[0]
    err = fp32_error_vs_fp64(g, small[0], small[1], small[2])
    return {"workload": "256 independent 2-D dam breaks, fluid counts log-uniform 2k-200k, aspect 0.5-4, "
                        "dx 0.005-0.02, alpha 0.005-0.05, delta 0.05-0.2 (seeded), FP32 pair arithmetic, "
                        "FP64 positions",
            "instances": tot["instances"], "particles": tot["particles"], "cells": tot["cells"],
            "value": value, "unit": "particle-steps/s", "timed_steps": args.batched_steps,
            "ms_per_step": ms / args.batched_steps, "admission_s": t_admit, "tuning": tuning,
            "list_skin": skin, "list_builds_in_timed_steps": builds,
            "kernel_ms_20_steps": fam,
            "plain_fp64_same_instances": {"value": plain, "unit": "particle-steps/s",
                                          "sample": "smallest, median and largest instance, each alone, 30 steps"},
            "ratio_vs_plain_fp64_same_instances": value / plain,
            "ratio_vs_plain_fp64_c1": value / plain_c1,
            "error_vs_fp64": err}


def run_serving(g, args):
    """The serving workload: Poisson arrivals (mean 20 req/s) of dam-break
    solves, 70% 2-D / 30% 3-D, particle counts log-uniform 5k-2M, horizons
    uniform 0.05-0.5 s scaled by --serving-horizon-scale, FP32 ensembles."""
    import numpy as np
    S = g.serving
    raw = g.workloads.serving_requests(args.serving_requests, horizon_scale=args.serving_horizon_scale)
    caps = tuple(int(c) for c in args.serving_caps.split(","))

    def serve(policy):
        reqs = [S.Request(i, t, g.spec_from_case(c), n) for i, (t, c, n) in enumerate(raw)]
        loop = S.ServingLoop(chunk=64, policy=policy, caps=caps)
        st = loop.run(reqs)
        loop.close()
        return st

    stats = serve(args.serving_policy)
    stats["policy"] = {"name": args.serving_policy, "caps_2d_3d": list(caps) if args.serving_policy == "shortest"
                       else None}
    other = "arrival" if args.serving_policy == "shortest" else "shortest"
    o = serve(other)
    stats["other_policy"] = {"name": other, "p50_s": o["p50_s"], "p99_s": o["p99_s"], "mean_s": o["mean_s"],
                             "particle_steps_per_s": o["particle_steps_per_s"]}
    # the same solves run alone, one after another, on the plain FP64 path:
    # each one's time from its size class's measured FP64 rate
    by_d = {2: [c for _, c, _ in raw if c.D == 2], 3: [c for _, c, _ in raw if c.D == 3]}
    rates = {}
    for D, cs in by_d.items():
        if cs:
            cs = sorted(cs, key=lambda c: c.N)
            rates[D] = plain_fp64_rate(g, [cs[len(cs) // 2]], steps=20)
    alone = np.array([c.N * n / rates[c.D] for _, c, n in raw])
    # sequential service in arrival order
    t, lat = 0.0, []
    for (arr, c, n), a in zip(raw, alone):
        t = max(t, arr) + a
        lat.append(t - arr)
    lat = np.array(lat)
    tot_ps = sum(c.N * n for _, c, n in raw)
    stats.update({
        "workload": f"{len(raw)} requests, Poisson 20 req/s, 70% 2-D / 30% 3-D, particle counts log-uniform "
                    f"5k-2M, horizons uniform 0.05-0.5 s x {args.serving_horizon_scale} (dt 1e-5)",
        "plain_fp64_alone": {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                             "particle_steps_per_s": tot_ps / alone.sum(),
                             "how": "each solve alone, in arrival order, at the FP64 path's measured rate for "
                                    "its dimension (median-size request of that dimension, 20 steps)"},
    })
    stats["throughput_ratio_vs_plain_fp64"] = stats["particle_steps_per_s"] / stats["plain_fp64_alone"][
        "particle_steps_per_s"]
    return stats


# the reference's published update! / partialupdate! medians on 200,000
# uniform 2-D points, cellsize = dist = 0.016 (README.md:64-91), hardware not stated
PUBLISHED_UPDATE_MS = 43.195
PUBLISHED_PARTIAL_MS = 42.673


def run_celllist(g, reps=10):
    """The cell-list workload alone: update! (binning + pair list + emit into
    the pairs array) and partialupdate! (pair search on the stale cells after
    jittering the points by U(-0.1, 0.1)·dist), FP64, on 200,000 uniform 2-D
    points (cellsize = dist = 0.016) and 4,000,000 uniform 3-D points
    (cellsize = dist = 0.008); median wall time of `reps` synchronous calls."""
    import numpy as np
    import torch
    out = {}
    for key, N, D, cs in (("2d_200k", 200_000, 2, 0.016), ("3d_4m", 4_000_000, 3, 0.008)):
        x = g.workloads.uniform_points(N, D)
        c = g.GPUCellList(tuple(x), (cs,) * D, cs)
        c.update()
        c.update()

        def timed(fn):
            ts = []
            for _ in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fn()
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            return 1e3 * statistics.median(ts)

        up = timed(c.update)
        pairs = c.pairsn
        rng = np.random.default_rng(7)
        for d in range(D):
            c.points[d].add_(torch.from_numpy(rng.uniform(-0.1, 0.1, N) * cs).to(c.points[d].device))
        part = timed(c.partialupdate)
        out[key] = {"points": N, "pairs": pairs, "update_ms": up, "partialupdate_ms": part,
                    "pairs_per_s_update": pairs / (up / 1e3)}
        c.close()
    out["2d_200k"]["published_update_ms"] = PUBLISHED_UPDATE_MS
    out["2d_200k"]["published_partialupdate_ms"] = PUBLISHED_PARTIAL_MS
    out["2d_200k"]["update_speedup_vs_published"] = PUBLISHED_UPDATE_MS / out["2d_200k"]["update_ms"]
    out["2d_200k"]["partialupdate_speedup_vs_published"] = PUBLISHED_PARTIAL_MS / out["2d_200k"]["partialupdate_ms"]
    out["note"] = "published medians from the reference's README, hardware not stated"
    return out


# the reference's published stepsolve!(prob, 1) median on its 2-D Dp0.02
# fixture with dist = H (test/devtest.jl:460-472), hardware not stated
PUBLISHED_STEPSOLVE1_MS = 5.193


def run_fixture(g, reps=50):
    """stepsolve!(prob, 1) on the reference's own 2-D Dp0.02 fixture (4,704
    fluid + 1,491 boundary particles, hydrostatic ρ, README parameters):
    median wall time of one synchronous call through the public API, next to
    the published figure; and the per-step time of stepsolve!(prob, 15)."""
    import torch
    fx = os.path.join(ROOT, "tests", "golden", "dambreak2d_dp002.npz")
    case = g.workloads.load_fixture(fx)
    system = g.GPUCellList(tuple(case.x), case.cellsize, case.dist)
    prob = g.SPHProblem(system, case.dx, case.h, case.H, g.WendlandC2(dim=2), case.rho, case.ptype, case.rho0,
                        case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL)
    for _ in range(5):
        prob.stepsolve(1)
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prob.stepsolve(1)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    one = 1e3 * statistics.median(ts)
    prob.stepsolve(15)
    prob.stepsolve(15)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(10):
        prob.stepsolve(15)
    torch.cuda.synchronize()
    per_step = 1e3 * (time.perf_counter() - t0) / 150
    prob.close()
    system.close()
    return {"workload": "reference fixture test/input Dp0.02 (2-D), dist = H", "particles": case.N,
            "stepsolve_1_ms": one, "published_stepsolve_1_ms": PUBLISHED_STEPSOLVE1_MS,
            "speedup_vs_published": PUBLISHED_STEPSOLVE1_MS / one, "stepsolve_15_ms_per_step": per_step,
            "note": "published median from test/devtest.jl, hardware not stated; one call = one synchronous "
                    "host round trip through the public API"}


def run_c3(args):
    """3-D dam break at scale: fluid block 1.0 x 2.0 (vertical) x 0.5 m at
    dx = 0.01 (1.0 M fluid) in a 4.0 x 3.0 x 1.0 m tank with 3 boundary
    layers, h = √3 dx, full physics (ν = 0.2, s = 0.05, DPC l₀ = 0.005,
    λ = 0.005, pmax = 36000, XSPH ε = 0.5, CSPM every 15 steps).  The FP32
    ensemble and the FP64 drop-in each advance it `--c3-steps` steps; the
    per-field relative L2 error of FP32 against FP64 and both rates."""
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as ge
    g = ge.load_package()
    case = g.workloads.dam_break_3d(dx=args.c3_dx)
    n = args.c3_steps
    N = case.N
    # FP32 ensemble
    ens = g.Ensemble(3)
    slot = ens.add(g.spec_from_case(case))
    ens.step(30)  # tuning (24 steps) + warm-up
    torch.cuda.synchronize()
    # a fresh instance for the measured run, so both start from the same state
    ens.remove(slot)
    slot = ens.add(g.spec_from_case(case))
    t0 = time.perf_counter()
    ens.step(n)
    torch.cuda.synchronize()
    t32 = time.perf_counter() - t0
    f32 = {f: ens.get(slot, f) for f in ("x", "v", "rho")}
    tuning = ens.tuning()
    ens.close()
    # FP64 drop-in
    system = g.GPUCellList(tuple(case.x), case.cellsize, case.dist)
    prob = g.SPHProblem(system, case.dx, case.h, case.H, g.WendlandC2(dim=3), case.rho, case.ptype, case.rho0,
                        case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL, g=case.g, s=case.s)
    for k, val in case.extra.items():
        setattr(prob, k, val)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prob.stepsolve(n)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    x64 = torch.stack(system.points).cpu().numpy()
    v64 = torch.stack(prob.v).cpu().numpy()
    r64 = prob.rho.cpu().numpy()
    err = {"rho": rel_l2(f32["rho"], r64), "rho_minus_rho0": rel_l2(f32["rho"] - case.rho0, r64 - case.rho0),
           "v": rel_l2(f32["v"], v64), "displacement": rel_l2(f32["x"] - case.x, x64 - case.x),
           "x": rel_l2(f32["x"], x64)}
    out = {"metric": "particle-steps/s", "workload": "3-D dam break at scale, full physics, FP32 ensemble vs "
                                                     "FP64 drop-in", "particles": N,
           "fluid": int((case.ptype == 2).sum()), "steps": n, "dx": args.c3_dx,
           "fp32": {"value": N * n / t32, "seconds": t32, "tuning": tuning},
           "fp64": {"value": N * n / t64, "seconds": t64},
           "ratio_fp32_vs_fp64": t64 / t32, "fp32_error_vs_fp64": err}
    print(json.dumps(out))
    return 0


def run_gb300(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    import __graft_entry__ as ge
    g = ge.load_package()
    L = g.load_library()
    case = make_case(g)
    D, N = case.D, case.N

    def new_problem():
        system = g.GPUCellList(tuple(case.x), case.cellsize, case.dist)
        prob = g.SPHProblem(system, case.dx, case.h, case.H, g.WendlandC2(dim=D), case.rho, case.ptype, case.rho0,
                            case.m0, case.dt, case.alpha, case.c0, case.gamma, case.delta, case.CFL)
        return system, prob

    system, prob = new_problem()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # ---------------- device-resident measurement (library timers off)
    for _ in range(args.warmup):
        prob.stepsolve(SUB)
    L.gcsph_timing_enable(0)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = g.launch_count()
    barrier()
    with Clocks(local) as clk:
        for i in range(args.steps):
            flush.fill_(float(i))
            starts[i].record()
            prob.stepsolve(SUB)
            ends[i].record()
        barrier()
    launches = g.launch_count() - launches0
    ms = sum(starts[i].elapsed_time(ends[i]) for i in range(args.steps))
    ms = max_over_ranks(ms)
    value = ws * N * SUB * args.steps / (ms / 1e3)
    # per-kernel-family timers: the same K bench steps again, instrumented
    # (event nodes between the kernels), so the timed run above stays clean
    L.gcsph_timing_enable(1)
    L.gcsph_timing_reset()
    prob.stepsolve(SUB)  # captures the instrumented graph outside the count
    L.gcsph_timing_reset()
    barrier()
    for i in range(args.steps):
        flush.fill_(float(i))
        prob.stepsolve(SUB)
    barrier()
    import ctypes as C
    fam = {}
    for tid in range(L.gcsph_timing_count()):
        n_ = C.c_int64(); t_ = C.c_double()
        L.gcsph_timing_get(tid, C.byref(n_), C.byref(t_))
        fam[L.gcsph_timing_name(tid).decode()] = (int(n_.value), float(t_.value))
    L.gcsph_timing_enable(0)
    # the roofline covers the pair-sum kernel (pass A, stage 1), the hottest single kernel; the
    # neighbour build is a family of six short kernels (its split is in kernel_ms)
    top = "stage1" if fam.get("stage1", (0, 0))[0] else max(fam, key=lambda k: fam[k][1])
    npairs = system.pairsn
    # ---------------- end-to-end through the public API with host buffers
    hx = torch.empty((D, N), dtype=torch.float64).pin_memory()
    hv = torch.empty((D, N), dtype=torch.float64).pin_memory()
    hr = torch.empty(N, dtype=torch.float64).pin_memory()
    hx.copy_(torch.from_numpy(case.x)); hv.zero_(); hr.copy_(torch.from_numpy(case.rho))
    system2, prob2 = new_problem()
    h2d = d2h = (2 * D + 1) * N * 8
    e_st = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    e_en = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]

    def e2e_step():
        for d in range(D):
            system2.points[d].copy_(hx[d], non_blocking=True)
            prob2.v[d].copy_(hv[d], non_blocking=True)
        prob2.rho.copy_(hr, non_blocking=True)
        prob2.stepsolve(SUB)
        for d in range(D):
            hx[d].copy_(system2.points[d], non_blocking=True)
            hv[d].copy_(prob2.v[d], non_blocking=True)
        hr.copy_(prob2.rho, non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    for i in range(args.steps):
        flush.fill_(float(i))
        e_st[i].record()
        e2e_step()
        e_en[i].record()
    barrier()
    ms_e2e = sum(e_st[i].elapsed_time(e_en[i]) for i in range(args.steps))
    ms_e2e = max_over_ranks(ms_e2e)
    e2e = ws * N * SUB * args.steps / (ms_e2e / 1e3)
    if rank != 0:
        return 0
    # ---------------- roofline of the dominant kernel family
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        peaks = json.load(open(peaks_path))
        hbm_peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        hbm_peak, peak_src = 6800.0, "fallback"
    nl, tms = fam[top]
    avg_s = tms / 1e3 / max(nl, 1)
    if top in ("stage1", "stage2"):
        alg = algorithmic_bytes_per_stage(case, npairs)
    else:
        alg = None
    achieved = (alg / avg_s / 1e9) if alg else None
    roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": (achieved / hbm_peak) if achieved else None,
            "traffic": PAIRA_STAGE1_DRAM_BYTES if top == "stage1" else None, "peak_source": peak_src,
            "avg_launch_us": avg_s * 1e6, "alg_bytes_per_launch": alg,
            "fp64_pipe_frac_ncu": PAIRA_STAGE1_FP64_PIPE if top == "stage1" else None,
            "note": "pair-once pass A is FP64-pipe bound (2 FP64 instr/cycle/SM on GB300, ncu: 78% of that "
                    "peak); its working set stays in L2, so the HBM fraction against the measured copy "
                    "bandwidth is small by construction; 'fp64' is the algorithmic-flop side of the roofline"}
    if top == "stage1":
        # the compute side: the reference's per-pair flops over the measured launch time, against
        # the FP64 peak of 2 DFMA (4 flops) per cycle per SM at the SM clock sampled under load
        try:
            xs = torch.stack([p_.detach() for p_ in system.points]).cpu().numpy()
            vs = torch.stack([p_.detach() for p_ in prob.v]).cpu().numpy()
            flops, kinds = algorithmic_flops_stage1(case, xs, vs)
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            mhz = clk.summary().get("sm_mhz") or 2070.0
            fp64_peak = 4.0 * sms * mhz * 1e6
            roof["fp64"] = {"achieved": flops / avg_s / 1e12, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                            "frac": flops / avg_s / fp64_peak, "flops_per_launch": flops, "pairs": kinds,
                            "peak_source": f"ncu DFMA peak_sustained 2/cycle/SM x {sms} SMs x {mhz:.0f} MHz",
                            "state": "pairs and branches counted at the state after the timed steps"}
        except Exception as e:  # noqa: BLE001
            roof["fp64"] = {"unavailable": f"{type(e).__name__}: {e}"}
    cpu = None
    if not args.no_cpu_baseline:
        try:
            from oracle import oracle as orc
            v, n, el = cpu_baseline(case, args.cpu_seconds, 1)
            cpu = {"value": v, "unit": "particle-steps/s", "cores": 1, "kind": "port",
                   "sample": f"{n} SPH steps of the same workload in {el:.1f} s, serial oracle"}
        except Exception as e:  # noqa: BLE001
            cpu = {"value": None, "unit": "particle-steps/s", "cores": 0, "kind": "port", "sample": f"failed: {e}"}
    out = {"metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": WORKLOAD, "particles": N, "pairs": npairs, "sph_steps_per_bench_step": SUB,
                      "l2": "flushed (256 MB write) between bench steps", "parallelism": f"replicas x{ws}"},
           "e2e": {"value": e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(),
           "kernel_ms": {k: {"launches": v[0], "total_ms": v[1]} for k, v in fam.items() if v[0]},
           "kernel_timing": "library event timers over a second, instrumented pass of the same K bench steps",
           "graphs": dict(zip(("captured", "replayed"), prob.graph_stats()))}
    if not args.no_celllist:
        try:
            out["published_fixture"] = run_fixture(g)
        except Exception as e:  # noqa: BLE001
            out["published_fixture"] = {"error": repr(e)}
        try:
            out["celllist"] = run_celllist(g)
        except Exception as e:  # noqa: BLE001
            out["celllist"] = {"error": repr(e)}
    if not args.no_batched:
        try:
            out["batched_fp32"] = run_batched(g, args, value / ws)
        except Exception as e:  # noqa: BLE001
            out["batched_fp32"] = {"error": repr(e)}
    if not args.no_serving:
        try:
            out["serving"] = run_serving(g, args)
        except Exception as e:  # noqa: BLE001
            out["serving"] = {"error": repr(e)}
    print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.c3:
        return run_c3(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
