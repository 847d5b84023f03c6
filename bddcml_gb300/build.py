"""Builds libbddcgpu.so in-tree: host C++ with g++, device code with nvcc for
sm_103a only, linked into one shared library exporting the C ABI declared in
include/bddcml_gb300.h."""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libbddcgpu.so")
BUILD = os.path.join(HERE, "_build")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-variable", "-Wno-sign-compare"]
NVFLAGS = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp"]

SOURCES = [
    ("bddc_host.cpp", "g++"),
    ("bddc_abi.cpp", "g++"),
    ("bddc_adaptive.cpp", "g++"),
    ("bddc_levels.cpp", "g++"),
    ("bddc_global.cpp", "g++"),
    ("bddc_device.cu", "nvcc"),
    ("bddc_noalloc.cu", "nvcc"),
    ("bddc_gradient.cu", "nvcc"),
]
HEADERS = ["bddc_internal.hpp", "bddc_kernels.cuh", "bddc_df.cuh", "bddc_setup_kernels.cuh",
           "bddc_pcg_kernels.cuh", "bddc_tc.cuh", "bddc_adaptive.cuh", "bddc_batch_kernels.cuh",
           "bddc_batch.cuh", "bddc_ozaki.cuh", "bddc_batch_tc.cuh"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "bddcml_gb300.h")]
    objs, procs = [], []
    for src, tool in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            if tool == "g++":
                cmd = ["g++"] + CXXFLAGS + ["-c", s, "-o", o]
            else:
                cmd = [_nvcc()] + NVFLAGS + ["-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + out.decode(errors="replace"))
    if force or _stale(OUT, objs):
        cmd = [_nvcc()] + GENCODE + ["-shared", "-Xcompiler", "-fopenmp", "-o", OUT] + objs + ["-lgomp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + " ".join(cmd) + "\n" + r.stdout.decode(errors="replace"))
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
