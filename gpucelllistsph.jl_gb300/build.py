"""Build libgcsph.so in-tree with nvcc for sm_103a (no cmake, no torch).

One translation unit per .cu file, compiled in parallel, then linked with
`nvcc -shared`.  The FP64 drop-in kernels are built with -fmad=false so every
expression rounds like the reference's Julia source (no FMA contraction).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgcsph.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# translation unit -> extra flags
UNITS = {
    "common.cu": [],
    "celllist.cu": ["-fmad=false"],
    "sph_step.cu": ["-fmad=false"],
    "sph_once.cu": [],
    "sph_pairs.cu": ["-fmad=false"],
    "ensemble.cu": [],
    "serving.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, u) for u in UNITS]


def _deps():
    return _sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")] + [
        os.path.join(HERE, "..", "include", "gcsph.h"), __file__]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    base = [cc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler",
            "-fvisibility=hidden", "-I", os.path.join(HERE, "..", "include")]

    def one(unit):
        obj = os.path.join(OUT, unit.replace(".cu", ".o"))
        cmd = base + UNITS[unit] + ["-c", os.path.join(CSRC, unit), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(one, list(UNITS)))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
