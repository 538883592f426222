"""Builds libswave.so (sm_103a) in-tree with nvcc, and the CPU oracle.

The CUDA translation units are compiled in parallel, one -gencode, with
--fmad=false so that device arithmetic follows the reference's operation
order exactly, and -ffp-contract=off for host code for the same reason.
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
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "libswave.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

CUDA_SOURCES = ["kernels.cu", "batch.cu", "runner.cu", "engine.cu", "rtmjob.cu", "fwi.cu", "noalloc.cu", "cnn.cu", "regularize.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-O2",
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libswave")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_library(force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "swave.h"))
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I", os.path.join(ROOT, "include"),
                         "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    if verbose:
        print("built", LIB)
    return LIB


CLI_DIR = os.path.join(PKG, "cli")
BINDIR = os.path.join(LIBDIR, "bin")
# Program name (as the reference names it) -> its source in cli/.
CLI_PROGRAMS = {
    "Acoustic_modeling_sep.x": "acoustic_modeling_sep.c",
    "3DRTM.x": "rtm3d.c",
    "3DBORNMOD.x": "bornmod3d.c",
    "2DAFWI.x": "afwi2d.c",
    "L_BFGS.x": "lbfgs.c",
}


def build_cli(force: bool = False) -> dict[str, str]:
    """Compiles the SEP command-line programs against libswave.so (host C;
    the library is found next to them through the run path)."""
    build_library()
    os.makedirs(BINDIR, exist_ok=True)
    common = [os.path.join(CLI_DIR, f) for f in ("sep.c", "swcli.c")]
    deps = common + [os.path.join(CLI_DIR, f) for f in ("sep.h", "swcli.h")] + [
        os.path.join(ROOT, "include", "swave.h"), LIB]
    cc = shutil.which("gcc") or "gcc"
    jobs, out = [], {}
    for exe, src in CLI_PROGRAMS.items():
        target = os.path.join(BINDIR, exe)
        out[exe] = target
        s = os.path.join(CLI_DIR, src)
        if force or _stale(target, [s] + deps):
            jobs.append([cc, "-O2", "-std=c11", "-Wall", "-Wextra", "-Wno-unused-parameter",
                         "-I", os.path.join(ROOT, "include"), "-o", target, s, *common,
                         "-L", LIBDIR, "-lswave", "-Wl,-rpath,$ORIGIN/..", "-lm"])
    sep_lib = os.path.join(LIBDIR, "libswsep.so")
    if force or _stale(sep_lib, common + deps[2:4]):
        jobs.append([cc, "-O2", "-std=c11", "-Wall", "-fPIC", "-shared", "-o", sep_lib,
                     common[0]])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    out["libswsep.so"] = sep_lib
    return out


def build_oracle(force: bool = False) -> str:
    """Compiles the CPU restatement used by the tests and the CPU baseline."""
    src = os.path.join(ORACLE_DIR, "swave_oracle.cpp")
    deps = [src, os.path.join(ORACLE_DIR, "oracle.h"), os.path.join(ROOT, "include", "swave.h")]
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    if force or _stale(ORACLE_LIB, deps):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              "-o", ORACLE_LIB, src])
    return ORACLE_LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    build_library(force=force, verbose=True)
    build_cli(force=force)
    build_oracle(force=force)
