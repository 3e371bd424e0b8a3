"""Compile ``libapple_gb300.so`` in-tree (nvcc for sm_103a, g++ for host code).

Translation units compile in parallel; the library is rebuilt only when a
source or header is newer than it.
"""

from __future__ import annotations

import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libapple_gb300.so"
INCLUDE = HERE.parent / "include"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", f"-I{CUDA_HOME}/include"]

CU_SOURCES = ["fem_eval.cu", "solver.cu", "fem_noalloc.cu", "adjoint.cu", "batch.cu"]
CXX_SOURCES = ["capi.cpp", "prep.cpp"]


def _deps() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*")) + sorted(INCLUDE.glob("*.h")) + [pathlib.Path(__file__)]


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        jobs.append([NVCC, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        jobs.append(["g++", *CXX_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    procs = [(cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for cmd in jobs]
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(" ".join(cmd))
    if failed:
        raise RuntimeError("apple_gb300 build failed:\n" + "\n".join(failed))
    tmp = LIB.with_suffix(".so.tmp")
    link = [NVCC, *GENCODE, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("apple_gb300 link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
