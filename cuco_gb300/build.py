"""Build libcuco_gb300.so for sm_103a with nvcc (no CMake).

Each CUDA translation unit in csrc/ compiles in parallel to an object, then one
nvcc link makes the shared library in cuco_gb300/_lib/.  The library is built
in-tree so that the process loading it is the one using it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libcuco_gb300.so")
SOURCES = ["sort.cu", "shortrange.cu", "pm.cu", "engine.cu", "capi_gpu.cu", "dropin.cu", "ensemble.cu",
           "sort_static.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
         "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


DEBUG_LIB = os.path.join(OUT, "libcuco_gb300_debug.so")


def build(verbose: bool = False, force: bool = False, extra_flags: list[str] | None = None,
          debug: bool = False) -> str:
    """The release library; with debug=True the debug build with the kernels'
    bounds checks (CUCO_BOUNDS_CHECK), libcuco_gb300_debug.so, beside it."""
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    cc = nvcc()
    flags = FLAGS + (extra_flags or []) + (["-DCUCO_BOUNDS_CHECK"] if debug else [])
    lib_path = DEBUG_LIB if debug else LIB
    suffix = ".debug.o" if debug else ".o"

    def compile_one(src: str) -> str:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + suffix)
        if not force and _newer(o, [s] + headers + [__file__]):
            return o
        cmd = [cc, *ARCH, *flags, "-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return o

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or not _newer(lib_path, objs):
        cmd = [cc, *ARCH, "-shared", "-o", lib_path, *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    return lib_path


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
