"""Builds libp9idg.so (CUDA kernels for sm_103a + the C ABI) in-tree with nvcc and g++.

Each translation unit compiles in parallel; objects are rebuilt only when a source
or header is newer.  The planner is host C++ compiled with -ffp-contract=off so its
floating-point expressions round exactly as the reference's C# does.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libp9idg.so")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _deps():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + _deps())


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
               "-c", src, "-o", obj]
        if ptxas_verbose:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((obj, src, cmd))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
               "-I", INCLUDE, "-c", src, "-o", obj]
        jobs.append((obj, src, cmd))
    todo = [j for j in jobs if ptxas_verbose or _stale(j[0], j[1])]
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        for out in ex.map(lambda j: _run(j[2], verbose), todo):
            logs.append(out)
    objs = [j[0] for j in jobs]
    if todo or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        libdir = os.path.join(home, "lib64")
        if not os.path.isdir(libdir):
            libdir = os.path.join(home, "lib")
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-L", libdir, "-lcufft", "-lpthread",
              "-Xlinker", f"-rpath,{libdir}"], verbose)
    return "\n".join(logs)


if __name__ == "__main__":
    import sys
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
    print(LIB)
