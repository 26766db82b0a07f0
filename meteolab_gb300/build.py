"""Builds libstormgpu.so (the device step and its C ABI) in-tree with nvcc for sm_103a only.

The translation units compile in parallel; the result lands next to this file as ``libstormgpu.so``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libstormgpu.so")
OBJDIR = os.path.join(HERE, "_build")
SOURCES = ["sg_kernels.cu", "sg_transport.cu", "sg_diag.cu", "sg_runtime.cu", "sg_static.cu", "sg_state.cu", "sg_electric.cu",
           "sg_lightning.cu", "sg_masked.cu"]
HEADERS = ["sg_common.cuh", "sg_device.cuh", "sg_fft.cuh", "sg_physics.cuh", "sg_kernels.h", "sg_state.h", "sg_tile_copies.cuh",
           "sg_charge.cuh", "sg_takahashi.h", "sg_elec_solve.cuh", "sg_lightning.h", "sg_rain2m.cuh", "sg_ice2m.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-Xptxas", "-v"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the device step needs the CUDA toolkit to build")
    return path


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    include = os.path.join(os.path.dirname(HERE), "include")
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(include, "stormgpu.h")]
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, deps + [s]):
            jobs.append([nvcc(), *ARCH, *FLAGS, "-I", include, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for log in ex.map(run, jobs):
            if verbose:
                print(log, file=sys.stderr)
    if force or _stale(LIB, objs):
        run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
