"""Builds libdepix.so (the C-ABI library) for sm_103a with nvcc.

Translation units compile in parallel into ``_build/``; the shared library
lands next to this file. No cmake, one -gencode, a minute or less.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdepix.so")
UNITS = ["depix_graph.cu", "depix_geom.cu", "depix_api.cu", "depix_queue.cu", "depix_refine.cu", "depix_static.cu",
         "depix_walks.cu"]
HEADERS = ["depix_device.cuh", "depix_internal.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(SRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "depix.h")]
    jobs = []
    for u in UNITS:
        src = os.path.join(SRC, u)
        obj = os.path.join(OUT_DIR, u.replace(".cu", ".o"))
        if _stale(obj, [src] + hdrs + [__file__]):
            jobs.append([nvcc, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
        return r

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(OUT_DIR, u.replace(".cu", ".o")) for u in UNITS]
    if jobs or _stale(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
