"""Builds libpicpp_gb300.so in-tree for sm_103a (GB300).

    python -m picpp_gb300.build        (or picpp_gb300.build.build())

Translation units compile in parallel with nvcc; the FP64 particle kernels
use --fmad=false so that their arithmetic rounds like the CPU oracle.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpicpp_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                 "--expt-relaxed-constexpr", "-I", os.path.join(HERE, os.pardir, "include"),
                 # register budget of the fused explicit kernel: CTAs per SM
                 f"-DPIC_TILE_MIN_BLOCKS={int(os.environ.get('PICPP_TILE_MIN_BLOCKS', '2'))}",
                 f"-DPIC_TILE_THREADS={int(os.environ.get('PICPP_TILE_THREADS', '512'))}",
                 f"-DPIC_IMP_THREADS={int(os.environ.get('PICPP_IMP_THREADS', '256'))}",
                 f"-DPIC_MOVER_THREADS={int(os.environ.get('PICPP_MOVER_THREADS', '256'))}"]
UNITS = {
    "api.cu": [],
    "solver.cu": [],
    "grid.cu": [],
    "kernels_f32.cu": [],
    "kernels_f64.cu": ["--fmad=false"],
    "energy_noalloc.cu": [],
    "init.cu": [],
    "nn.cu": [],
}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_mtime() -> float:
    m = 0.0
    for root in (CSRC, os.path.join(HERE, os.pardir, "include")):
        for f in os.listdir(root):
            m = max(m, os.path.getmtime(os.path.join(root, f)))
    return m


def _compile(unit: str, extra: list[str], verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    cmd = [nvcc()] + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
