"""Build the native libraries in-tree.

* libsdbf_gb300.so -- CUDA kernels for sm_103a + host orchestration + C ABI
  (include/sdbf_gb300.h) + SDBF text codec.
* libsdbf_synth.so -- seeded synthetic workload generator (plain C).

Translation units compile in parallel; a library is rebuilt only when one of
its sources is newer than it.  Run ``python -m sdhash_gb300.build``.
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
LIB = os.path.join(HERE, "libsdbf_gb300.so")
SYNTH = os.path.join(HERE, "libsdbf_synth.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = os.environ.get("SDBFG_ARCH", "-gencode=arch=compute_103a,code=sm_103a")
CU_SOURCES = ["gen_kernels.cu", "compare_kernels.cu", "matrix_tc.cu", "sdbf_api.cu", "compare_api.cu", "serve.cu",
              "noalloc.cu", "text_load.cu",
              "index_search.cu"]
CPP_SOURCES = ["sdbf_text.cpp", "../compat/sdbf_compat.cpp"]
HEADERS = ["gen_kernels.h", "compare_kernels.h", "compare_device.cuh", "ctx_internal.h", "matrix_plan.h", "sdbf_device.cuh", "sdbf_tables.h", "../compat/sdbf_class.h",
           "../compat/sdbf_set.h", "../compat/sdbf_conf.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_gb300(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "sdbf_gb300.h")]
    objs, jobs = [], []
    for src in CU_SOURCES + CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            if src.endswith(".cu"):
                cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                       "-I", CSRC, "-c", s, "-o", o]
            else:
                cmd = [nvcc, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-I", CSRC,
                       "-x", "c++", "-c", s, "-o", o]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"])
        if verbose:
            print("built", LIB)
    return LIB


def build_synth(force: bool = False) -> str:
    src = os.path.join(CSRC, "synth.c")
    if force or _stale(SYNTH, [src]):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-shared", "-o", SYNTH, src, "-lm", "-lpthread"])
    return SYNTH


CLI_SRC = os.path.join(HERE, "cli", "sdhash_main.cpp")
CLI = os.path.join(HERE, "sdhash-gb300")


def build_cli(force: bool = False) -> str:
    """The native command line (sdhash's options) linked against the library."""
    lib = build_gb300()
    if force or _stale(CLI, [CLI_SRC, lib, os.path.join(INCLUDE, "sdbf_gb300.h")]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", "-Wall", "-o", CLI, CLI_SRC, "-L", HERE, "-lsdbf_gb300",
              "-Wl,-rpath,$ORIGIN", "-lpthread"])
    return CLI


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_synth(force)
    build_gb300(force, verbose)
    build_cli(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
