"""Build libmrmd_gb300.so (CUDA kernels + C ABI) for sm_103a, in-tree.

Each translation unit under csrc/ is compiled by nvcc in parallel and the
objects are linked into ``mrmd_gb300/libmrmd_gb300.so``.  Objects are reused
when they are newer than their source and every header.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libmrmd_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
    "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}",
    # double4 is deprecated in CUDA 13 in favour of explicitly aligned types
    "-Xcudafe", "--diag_suppress=1444", "-Xcompiler", "-Wno-deprecated-declarations",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


# The bounds-checked debug build (-DMRMD_BOUNDS_CHECK: every kernel index into
# a particle, cell or list array is checked, see MRMD_IN_BOUNDS) goes to its
# own object folder and library, loaded when MRMD_GB300_BOUNDS_CHECK=1.
OBJ_BOUNDS = os.path.join(PKG, "_build_bounds")
LIB_BOUNDS = os.path.join(PKG, "libmrmd_gb300_bounds.so")


def _compile(src: str, extra: list[str], objdir: str = OBJ) -> str:
    obj = os.path.join(objdir, os.path.basename(src).replace(".cu", ".o"))
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest and (not extra or objdir != OBJ):
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


CPP_INCLUDE = os.path.join(PKG, "cpp", "include")
CPP_EXAMPLES = os.path.join(PKG, "cpp", "examples")


def build_examples() -> list[str]:
    """Compile the C++ drivers written against the drop-in headers."""
    outs = []
    for src in sorted(glob.glob(os.path.join(CPP_EXAMPLES, "*.cpp"))):
        exe = os.path.join(OBJ, os.path.basename(src)[:-4])
        deps = [src, LIB] + glob.glob(os.path.join(CPP_INCLUDE, "**", "*.hpp"), recursive=True)
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(d) for d in deps):
            outs.append(exe)
            continue
        # mrmd/ on the include path too: drivers written against the reference
        # include "action/LennardJones.hpp" and the like
        cmd = ["g++", "-O2", "-std=c++20", "-Wall", f"-I{INCLUDE}", f"-I{CPP_INCLUDE}",
               f"-I{os.path.join(CPP_INCLUDE, 'mrmd')}", src, "-o", exe,
               f"-L{PKG}", "-lmrmd_gb300", f"-Wl,-rpath,{PKG}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for {src}:\n{r.stdout}\n{r.stderr}")
        outs.append(exe)
    return outs


def build(verbose: bool = False, extra: list[str] | None = None, bounds_check: bool = False) -> str:
    objdir, lib = (OBJ_BOUNDS, LIB_BOUNDS) if bounds_check else (OBJ, LIB)
    os.makedirs(objdir, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = list(extra or []) + (["-DMRMD_BOUNDS_CHECK"] if bounds_check else [])
    with cf.ThreadPoolExecutor(max_workers=min(16, len(sources))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, objdir), sources))
    stale = not (os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(o) for o in objs))
    if stale or (extra and not bounds_check):
        tmp = lib + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
        if verbose:
            print(f"built {lib}")
    if not bounds_check:
        build_examples()
    return lib


if __name__ == "__main__":
    args = sys.argv[1:]
    bounds = "--bounds-check" in args
    print(build(verbose=True, extra=[a for a in args if a != "--bounds-check"], bounds_check=bounds))
