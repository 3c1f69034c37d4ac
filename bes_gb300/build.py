"""Build the native library libbes_gb300.so in-tree (bes_gb300/_build/).

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host C++ units go through the same nvcc driver
(g++ underneath).  Units compile in parallel; a unit is rebuilt when it or any header in csrc/
or include/ is newer than its object.

    python -m bes_gb300.build [--force] [--ptxas-verbose]
"""
from __future__ import annotations

import argparse
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbes_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build bes_gb300")


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _compile(src: str, obj: str, verbose_ptxas: bool) -> str:
    # host code without FMA contraction, so that x86 and Arm hosts compute the same geometry
    flags = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
             "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-pthread",
             "-I" + os.path.join(ROOT, "include")]
    if src.endswith(".cu"):
        flags += ARCH + ["-lineinfo", "--expt-relaxed-constexpr"]
        if verbose_ptxas:
            flags += ["-Xptxas", "-v"]
    cmd = [nvcc()] + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose_ptxas: bool = False, quiet: bool = True) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    newest_header = max((os.path.getmtime(h) for h in _headers()), default=0.0)
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s),
                                                                         newest_header):
            jobs.append((s, o))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(lambda j: _compile(j[0], j[1], verbose_ptxas), jobs))
        if not quiet or verbose_ptxas:
            for (s, _), out in zip(jobs, outs):
                if out.strip():
                    print(f"== {os.path.basename(s)}\n{out}", file=sys.stderr)
    if (jobs or not os.path.exists(LIB)
            or max(os.path.getmtime(o) for o in objs) > os.path.getmtime(LIB)):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-pthread", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose_ptxas=a.ptxas_verbose, quiet=False))
