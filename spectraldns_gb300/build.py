"""Build the C-ABI shared library ``libsdns_gb300.so`` in-tree for sm_103a.

Each CUDA translation unit is compiled by its own ``nvcc`` process (in
parallel), then linked with the CUDA runtime into
``spectraldns_gb300/lib/libsdns_gb300.so``.  Run ``python -m
spectraldns_gb300.build`` or call :func:`build`.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "lib", "_obj")
LIBNAME = "libsdns_gb300.so"

SOURCES = [
    "sdns_kernels_f32.cu",
    "sdns_kernels_f64.cu",
    "sdns_capi.cu",
    "sdns_noalloc.cu",
    "sdns_les.cu",
    "sdns_pad32.cu",
]
EXTRA_SOURCES: list = []  # appended by later modules (LES closure kernels)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "sdns_gb300.h"))
    srcs = SOURCES + [s for s in EXTRA_SOURCES if s not in SOURCES]
    jobs = []
    objs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJDIR, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _newer(obj, [src] + headers):
            jobs.append([nvcc()] + ARCH + FLAGS + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-6000:]))
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out:
                print(out)
    lib = lib_path()
    if force or jobs or _newer(lib, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-cudart", "static"]
        run(cmd)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
