"""In-tree build of the engine's shared library (libxgm.so) for sm_103a, and of the
command-line front end xgm_count_cli (cli/xgm_count_cli.cpp, C ABI only).

Every translation unit under csrc/ is compiled by nvcc in parallel and linked into
x-gminer_gb300/libxgm.so with the CUDA runtime linked statically, so the library loads
with no CUDA path set.  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libxgm.so")
CLI_SRC = os.path.join(HERE, "cli", "xgm_count_cli.cpp")
CLI = os.path.join(HERE, "xgm_count_cli")
INCLUDE = os.path.join(HERE, "..", "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no floating-point contraction, so the seeded generators give the same
# samples on x86-64 and aarch64
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, f))
    return out


def _headers_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(src: str, obj: str) -> None:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for src in _sources():
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr):
            jobs.append((src, obj))
    if jobs:
        workers = min(len(jobs), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(workers) as ex:
            for f in [ex.submit(_compile, s, o) for s, o in jobs]:
                f.result()
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    _build_cli(relink=bool(jobs), hdr=hdr)
    if verbose:
        print(f"built {LIB} ({len(jobs)} units recompiled)", file=sys.stderr)
    return LIB


def _build_cli(relink: bool, hdr: float) -> None:
    """xgm_count_cli next to libxgm.so (found through an $ORIGIN rpath)."""
    if (not relink and os.path.exists(CLI)
            and os.path.getmtime(CLI) >= max(os.path.getmtime(CLI_SRC), hdr)):
        return
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for xgm_count_cli")
    tmp = CLI + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-I", INCLUDE, CLI_SRC, "-L", HERE, "-lxgm",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"xgm_count_cli build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)


if __name__ == "__main__":
    build(verbose=True)
