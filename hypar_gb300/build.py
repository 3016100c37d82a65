"""Build libgbhypar.so (and the gbhypar command-line driver) in-tree.

CUDA sources are compiled by nvcc for sm_103a only; the C host shell by gcc.
Translation units compile in parallel; outputs go next to this file
(git-ignored).  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbhypar.so")
CLI = os.path.join(HERE, "gbhypar")

CU_SOURCES = ["gbh_hyp_e1.cu", "gbh_hyp_e2.cu", "gbh_hyp_ns.cu", "gbh_hyp_e1w.cu", "gbh_hyp_e2w.cu", "gbh_hyp_nsw.cu", "gbh_hyp_nsg.cu", "gbh_hyp_e1b.cu", "gbh_hyp_e2b.cu", "gbh_hyp_nsb.cu", "gbh_visc.cu", "gbh_api.cu", "gbh_probe.cu", "gbh_ensemble.cu",
              "gbh_noalloc.cu", "gbh_adjoint.cu", "gbh_monitor.cu", "gbh_crweno.cu"]
C_SOURCES = ["gbh_inputs.c", "gbh_run.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_nvcc=None) -> str:
    """Compile every translation unit and link libgbhypar.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "gbhypar.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", CSRC,
                                   "-I", INCLUDE, "-c", s, "-o", o]
            if extra_nvcc:
                cmd[1:1] = list(extra_nvcc)
            jobs.append(cmd)
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".c", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["gcc", "-O2", "-std=c99", "-fPIC", "-Wall", "-I", INCLUDE, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(os.cpu_count() or 8, 16, len(jobs)))) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", LIB] + objs)
    main_src = os.path.join(CSRC, "gbhypar_main.c")
    if force or _stale(CLI, [main_src, LIB]):
        _run(["gcc", "-O2", "-std=c99", "-I", INCLUDE, "-o", CLI, main_src, "-L", HERE, "-lgbhypar",
              "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
