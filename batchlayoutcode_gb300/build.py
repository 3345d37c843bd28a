"""Build the GB300 BatchLayout engine in-tree.

    python -m batchlayoutcode_gb300.build

Produces, under batchlayoutcode_gb300/_build/ (git-ignored):
  libbatchlayout_gb300.so   CUDA kernels (sm_103a) + host code + the C ABI
  batchlayout               the command-line tool (same flags as the reference CLI)

Every translation unit is compiled in parallel; nvcc gets one -gencode.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libbatchlayout_gb300.so")
CLI = os.path.join(OUT, "batchlayout")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["minibatch.cu", "greedy.cu", "bfsinit.cu", "barnes_hut.cu", "batched.cu", "mpnn.cu", "features.cu", "learned.cu", "reduce.cu", "waits.cu", "api.cu"]
CPP_SOURCES = ["host.cpp"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd, log: str | None = None):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if log:
        with open(log, "w") as f:
            f.write(r.stdout)
    return r.stdout


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    """Compile what changed.  Each CUDA unit's ptxas resource report
    (registers, spills, shared memory per kernel) is kept beside its object
    as <unit>.ptxas.txt."""
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "batchlayout_gb300.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers) or not os.path.exists(o[:-2] + ".ptxas.txt"):
            jobs.append(([nv, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas=-v",
                          "--expt-relaxed-constexpr", "-c", s, "-o", o], o[:-2] + ".ptxas.txt"))
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if _newer(o, [s] + headers):
            jobs.append((["g++", "-O2", "-std=c++17", "-fPIC", "-c", s, "-o", o], None))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        outs = list(ex.map(lambda j: _run(*j), jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if _newer(LIB, objs):
        _run([nv, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    cli_src = os.path.join(PKG, "cli", "batchlayout.cpp")
    if os.path.exists(cli_src) and _newer(CLI, [cli_src, LIB] + headers):
        _run(["g++", "-O2", "-std=c++17", "-o", CLI, cli_src, "-I" + os.path.join(ROOT, "include"),
              "-I" + CSRC, "-L" + OUT, "-lbatchlayout_gb300", "-Wl,-rpath," + OUT])
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    print(LIB)
