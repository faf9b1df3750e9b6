"""In-tree build of libdg3d.so (and the dg3d driver) for sm_103a.

Compiles every CUDA/C++ translation unit of csrc/ in parallel with nvcc / g++
and links lib/libdg3d.so; the driver executable bin/dg3d links against it.
Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(PKG, "lib", "libdg3d.so")
BIN = os.path.join(PKG, "bin", "dg3d")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + INCLUDE, "-I" + CSRC]

LIB_CU = ["dg_solver.cu", "dg_noalloc.cu", "batch.cu", "serve.cu"]
LIB_CPP = ["basis.cpp", "mesh.cpp", "params.cpp", "h5lite.cpp", "snapshot.cpp"]
DRIVER_CPP = ["host/Basis.cpp", "host/Grid.cpp", "host/HDF5Functions.cpp", "host/driver.cpp"]


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _newest_header() -> float:
    hs = glob.glob(os.path.join(CSRC, "**", "*.h"), recursive=True) + glob.glob(
        os.path.join(CSRC, "**", "*.cuh"), recursive=True) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src: str, verbose: bool) -> str:
    rel = os.path.relpath(src, CSRC).replace(os.sep, "_")
    obj = os.path.join(OBJ, rel + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _newest_header()):
        return obj
    cuda_inc = os.path.join(_cuda_home(), "include")
    if src.endswith(".cu"):
        cmd = ["nvcc"] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I" + cuda_inc, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(verbose: bool = False, driver: bool = True) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    srcs = [os.path.join(CSRC, f) for f in LIB_CU + LIB_CPP]
    drv = [os.path.join(CSRC, f) for f in DRIVER_CPP] if driver else []
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
        dobjs = list(ex.map(lambda s: _compile(s, verbose), drv))
    if (not os.path.exists(LIB)) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = ["nvcc"] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    if driver and ((not os.path.exists(BIN)) or os.path.getmtime(BIN) < max(
            [os.path.getmtime(o) for o in dobjs] + [os.path.getmtime(LIB)])):
        cmd = ["g++", "-o", BIN] + dobjs + ["-L" + os.path.dirname(LIB), "-ldg3d",
                                           "-Wl,-rpath,$ORIGIN/../lib", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv))
