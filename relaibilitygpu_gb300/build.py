"""Build recipe for the engine: libnr.so (C ABI) and the network_reliability CLI.

Everything is compiled in-tree with nvcc for sm_103a only; translation units
are compiled in parallel.  The CPU oracle (test infrastructure) is built by
its own Makefile under oracle/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnr.so")
CLI = os.path.join(PKG, "network_reliability")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC]

CU_SOURCES = ["nr_api.cu", "nr_engine_g8.cu", "nr_engine_g16.cu", "nr_engine_g32.cu", "nr_engine_wide.cu",
              "nr_engine_wide_learn.cu", "nr_engine_wide_multi.cu", "nr_engine_wide_lanes.cu",
              "nr_engine_lane.cu", "nr_engine_block.cu", "nr_mlp.cu", "nr_noalloc.cu", "nr_io.cu", "nr_batch.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hdrs + [os.path.join(INCLUDE, "nr.h")]


def build(verbose: bool = False, force: bool = False, extra_flags=None) -> str:
    """Compile libnr.so and the CLI if any source is newer than the outputs."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = NVCC_FLAGS + list(extra_flags or [])
    hdrs = _deps()
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([cc] + ARCH + flags + ["-c", s, "-o", o])
    log = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                log.append(out)
    if force or jobs or _stale(LIB, objs):
        log.append(_run([cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]))
    cli_src = os.path.join(CSRC, "nr_cli.cpp")
    if force or _stale(CLI, [cli_src, LIB, os.path.join(INCLUDE, "nr.h")]):
        log.append(_run([cc] + ARCH + ["-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", CLI,
                                       "-L" + PKG, "-lnr", "-Xlinker", "-rpath=$ORIGIN"]))
    text = "".join(log)
    if verbose and text:
        sys.stdout.write(text)
    return text


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv,
          extra_flags=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None)
