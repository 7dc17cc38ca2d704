"""Build of liblighter_gb300.so (nvcc, sm_103a only) and of the CPU oracle.

The translation units compile in parallel; the library links the CUDA
runtime statically so it only needs the driver at run time. Everything lands
in-tree (git-ignored): lighter_gb300/_build/*.o, lighter_gb300/liblighter_gb300.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblighter_gb300.so")

SOURCES = ["api.cpp", "bake.cu", "bvh.cu", "radiosity.cu", "reftree.cpp", "noalloc.cu", "gather.cu", "rng.cpp",
           "trace.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false (device) and -ffp-contract=off (host; aarch64 g++ contracts by
# default) keep a*b+c as two roundings, like the reference's CPU build,
# so the arithmetic-only stages reproduce it bit for bit.
NVFLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
                  "-DLTRBUILD", "-diag-suppress", "550"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVFLAGS + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fPIC", "-lpthread"])
    return LIB


def build_oracle() -> None:
    """CPU checkers: the oracle port always; the reference build only where
    its sources are present (oracle/Makefile decides)."""
    _run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"])


if __name__ == "__main__":
    print(build_library(verbose=True))
    build_oracle()
