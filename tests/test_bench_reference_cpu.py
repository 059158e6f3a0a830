"""The bench's reference arm on CPU: one JSON line with the contract's keys,
the reference's CPU restatement timed on the host cores."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, lines
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"] and d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_pass_a_flop_count_by_hand():
    """The roofline's flop side on a configuration counted by hand (2-D): two
    fluid particles approaching each other, a boundary (ptype 0) particle
    within r0 = 2dx of one of them, and a second boundary particle that pairs
    only with the first boundary particle."""
    import types
    import numpy as np
    b = _bench_module()
    dx = 0.1
    case = types.SimpleNamespace(D=2, dx=dx, dist=0.25, ptype=np.array([2, 2, 0, 0], dtype=np.int32))
    x = np.array([[0.0, 0.2, -0.05, -0.05], [0.0, 0.0, -0.14, -0.37]])
    v = np.array([[1.0, -1.0, 0.0, 0.0], [0.0, 0.0, 0.0, 0.0]])
    flops, kinds = b.algorithmic_flops_stage1(case, x, v)
    # pairs: (0,1) fluid-fluid at 0.2, approaching; (0,2) fluid-boundary at 0.149 < 2dx;
    # (2,3) boundary-boundary at 0.23; (1,2) at 0.287 is past dist
    assert kinds == {"pairs": 3, "real": 1, "one_side_real": 1, "approaching": 1, "within_r0": 1}
    D = 2
    geometry = 7 * D + 16                                   # every pair
    ff = (7 * D + 1) + 2 * 34 + (3 * D + 4) + 3 * D + (5 * D + 10)
    fb_in = (3 * D + 1) + (3 * D + 14)
    assert flops == 3 * geometry + ff + fb_in == 236


def test_clock_record_reads_the_sampler_output(tmp_path):
    """The bench's clock record from the nvidia-smi sampler's CSV (no GPU): the
    median SM clock, the maximum, the number of samples and every throttle
    reason seen active in any sample."""
    bench = _bench_module()
    clk = bench.Clocks(0)
    clk.path = str(tmp_path / "clocks.csv")
    rows = [
        "0, 2070, 2070, 612.3, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 640.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 655.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    open(clk.path, "w").write("\n".join(rows) + "\n")
    s = clk.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    clk.path = str(tmp_path / "missing.csv")
    assert clk.summary()["reasons"] == ["unsampled"]
