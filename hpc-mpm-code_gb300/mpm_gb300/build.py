"""In-tree build of the CUDA library (libmpm_gb300.so) for sm_103a.

Every .cu file under csrc/ is compiled by its own nvcc process (in parallel)
with one -gencode for sm_103a, then linked into lib/libmpm_gb300.so.  Objects
are rebuilt only when a source or header is newer.  No cmake, no torch
extension machinery: the product is a plain C-ABI shared library.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
LIBDIR = os.path.join(PKG, "lib")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(LIBDIR, "libmpm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose=False, ptxas_info=False):
    obj = os.path.join(LIBDIR, os.path.basename(src) + ".o")
    deps = [src] + _headers()
    if not _stale(obj, deps):
        return obj, ""
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


DRIVER = os.path.join(LIBDIR, "explicit_driver")
SCENE_TOOL = os.path.join(LIBDIR, "scene_tool")


def build_host(verbose: bool = False) -> str:
    """The C++ host layer (host/gpu_solid.cpp, host/scene_io.cpp), its explicit
    driver and scene_tool, linked against libmpm_gb300.so.  Returns the driver."""
    lib = build(verbose)
    layer = [os.path.join(HOST, "gpu_solid.cpp"), os.path.join(HOST, "scene_io.cpp")]
    headers = [os.path.join(HOST, "gpu_solid.h"), os.path.join(HOST, "scene_io.h"), os.path.join(INCLUDE, "mpm_gpu.h")]
    for exe, main in ((DRIVER, "explicit_driver.cpp"), (SCENE_TOOL, "scene_tool.cpp")):
        srcs = layer + [os.path.join(HOST, main)]
        if _stale(exe, srcs + headers + [lib]):
            cmd = ["g++", "-O2", "-std=c++17", "-I" + INCLUDE, "-I" + HOST] + srcs + [
                "-L" + LIBDIR, "-lmpm_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe]
            if verbose:
                print(" ".join(cmd), flush=True)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"host build failed:\n{r.stdout}\n{r.stderr}")
    return DRIVER


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, ptxas_info), srcs))
    objs = [o for o, _ in results]
    if ptxas_info:
        for _, log in results:
            sys.stderr.write(log)
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
