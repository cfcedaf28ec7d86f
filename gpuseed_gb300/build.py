"""Builds libgpuseed.so (CUDA for sm_103a + the C-ABI) and the seed_gen CLI in-tree.

Translation units compile in parallel with nvcc into gpuseed_gb300/_build/ and
link into gpuseed_gb300/libgpuseed.so; seed_gen links against it with an
$ORIGIN rpath.  Rebuilds only what is older than its sources.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgpuseed.so")
CLI = os.path.join(PKG, "seed_gen")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-Wall",
                     "-I", INCLUDE]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgpuseed.so")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build(verbose: bool = False) -> str:
    """Compiles every CUDA translation unit and links libgpuseed.so and seed_gen."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    for src in sorted(glob.glob(os.path.join(CSRC, "gs_*.c"))):
        obj = os.path.join(BUILD, os.path.basename(src)[:-2] + ".c.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([cc, "-O2", "-std=gnu11", "-fPIC", "-Wall", "-pthread", "-ffp-contract=off",
                         "-I", INCLUDE, "-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and r.stderr:
                    print(r.stderr)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-pthread"])
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "seed_gen.c")
    if _stale(CLI, [cli_src, LIB] + headers):
        _run([cc, "-O2", "-std=gnu11", "-Wall", "-pthread", cli_src, "-o", CLI, "-I", INCLUDE, "-L", PKG,
              "-lgpuseed", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
