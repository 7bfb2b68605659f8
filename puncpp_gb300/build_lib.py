"""Compile libpunc_gpu.so in-tree for sm_103a.

Device translation units are built with --fmad=false (FP64 particle path in
the reference's rounding order); host code with -ffp-contract=off for the
same reason.  Units compile in parallel, then one nvcc link.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpunc_gpu.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC,
             "-I/usr/local/cuda/include"]

# unit -> extra nvcc flags
CU_UNITS = {
    "engine.cu": [],
    "k_particles.cu": [],
    "k_solver.cu": [],
    "k_inject.cu": [],
    "k_mixed.cu": ["--fmad=true"],
    "k_noalloc.cu": [],
    "k_amg.cu": [],
    "k_esolve.cu": ["--fmad=true"],
    "k_diag.cu": [],
    "k_step.cu": [],
    "k_adjoint.cu": [],
}
CPP_UNITS = ["mesh_tables.cpp", "amg.cpp", "checkpoint.cpp"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _sources_newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "punc_gpu.h"))
    jobs = []
    objs = []
    for unit, extra in CU_UNITS.items():
        src = os.path.join(CSRC, unit)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, unit + ".o")
        objs.append(obj)
        flags = [f for f in NVCC_FLAGS if not (extra and f.startswith("--fmad"))] + extra
        if force or _sources_newer(obj, [src] + headers):
            jobs.append([_nvcc()] + ARCH + flags + ["-c", src, "-o", obj])
    for unit in CPP_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit + ".o")
        objs.append(obj)
        if force or _sources_newer(obj, [src] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                if o.strip():
                    print(o)
    if force or jobs or _sources_newer(LIB, objs):
        _run([_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
