"""Build recipe of libemfa_cuda.so (sm_103a) and the C++ host front end.

Compiles every translation unit under csrc/ with nvcc in parallel
(-gencode arch=compute_103a,code=sm_103a) and links an in-tree shared
library, emfa_gb300/_build/libemfa_cuda.so.  No CMake, no torch extension
machinery: plain nvcc, so the same recipe runs on x86 and on the Arm GPU host.
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
LIB = os.path.join(BUILD, "libemfa_cuda.so")
LAUNCHER = os.path.join(BUILD, "emfa_launcher")
HOST = os.path.join(CSRC, "host")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FP contraction so host-side geometry/incidence math rounds
# like the reference's (x86 has no FMA in its baseline ISA; aarch64 does)
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
PER_FILE = {"geom.cu": ["-fmad=false"]}


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *NVFLAGS, *PER_FILE.get(src, []), "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr))
    if verbose and r.stderr:
        print(r.stderr, file=sys.stderr)
    return obj


def _stale(objs) -> bool:
    if not os.path.exists(LIB) or not os.path.exists(LAUNCHER):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(LAUNCHER))
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HOST, f) for f in os.listdir(HOST)]
    deps.append(os.path.join(HERE, "..", "include", "emfa_cuda.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def _build_launcher() -> None:
    """C++ host front end (solver classes + launcher) linked against the library."""
    srcs = [os.path.join(HOST, f) for f in sorted(os.listdir(HOST)) if f.endswith(".cpp")]
    cxx = shutil.which("g++") or "c++"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", *srcs, "-o", LAUNCHER, "-L" + BUILD, "-lemfa_cuda",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host front end build failed:\n" + r.stderr)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    if not force and not _stale(srcs):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    _build_launcher()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
