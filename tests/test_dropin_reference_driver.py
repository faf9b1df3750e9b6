"""The reference's own driver (cppsrc/driver.cpp) compiled and linked,
unchanged, against this package's C++ class facade (3ddg_gb300/csrc/host/)
and libdg3d.so: the drop-in claim that a user keeps their driver and swaps the
classes.  The driver file is copied into a temporary directory at test time
(never committed) from the reference's source directory that oracle/Makefile
names (or DG3D_REFERENCE_SRC); the test is skipped where that is absent.

Two builds: as shipped (float parameters, the Grid constructor taking
float*), and with FP64 parameters through the facade's pre-include
fp64_params.h (the double Grid constructor), the way the reference's FP64
build promotes float.  The linked executables are run on the paths that need
no GPU: a wrong argument count (exit code 1) and an unreadable parameter file
(exit code 3), the reference's error codes (cppsrc/driver.cpp:41-45).  CPU
only."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

HOST = os.path.join(ROOT, "3ddg_gb300", "csrc", "host")
LIB = os.path.join(ROOT, "3ddg_gb300", "lib")
FACADE = ["Basis.cpp", "Grid.cpp", "HDF5Functions.cpp"]


def reference_src():
    d = os.environ.get("DG3D_REFERENCE_SRC")
    if not d:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"], capture_output=True,
                           text=True)
        d = r.stdout.strip()
    return d


REF = reference_src()
pytestmark = pytest.mark.skipif(not (REF and os.path.isfile(os.path.join(REF, "driver.cpp"))),
                                reason="reference sources not present")


def cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def cxx(args, cwd):
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-w"] + args, cwd=cwd, capture_output=True, text=True)
    assert r.returncode == 0, "g++ %s\n%s\n%s" % (" ".join(args), r.stdout, r.stderr)


@pytest.fixture(scope="module")
def facade_objects(tmp_path_factory):
    import importlib
    importlib.import_module("3ddg_gb300.build").build(driver=False)
    d = tmp_path_factory.mktemp("facade")
    inc = ["-I" + HOST, "-I" + os.path.join(ROOT, "include"), "-I" + cuda_include()]
    objs = []
    for f in FACADE:
        o = str(d / (f + ".o"))
        cxx(inc + ["-c", os.path.join(HOST, f), "-o", o], str(d))
        objs.append(o)
    return objs


def build_reference_driver(tmp_path, facade_objects, fp64):
    shutil.copy(os.path.join(REF, "driver.cpp"), tmp_path / "driver.cpp")
    inc = ["-I" + HOST, "-I" + os.path.join(HOST, "single_process"), "-I" + os.path.join(ROOT, "include")]
    pre = ["-include", os.path.join(HOST, "fp64_params.h")] if fp64 else []
    cxx(inc + pre + ["-c", "driver.cpp", "-o", "driver.o"], str(tmp_path))
    cxx(["-o", "driver", "driver.o"] + facade_objects + ["-L" + LIB, "-ldg3d", "-Wl,-rpath," + LIB, "-lpthread"],
        str(tmp_path))
    und = subprocess.run(["nm", "-C", "-u", "driver.o"], cwd=tmp_path, capture_output=True, text=True).stdout
    return str(tmp_path / "driver"), und


@pytest.mark.parametrize("fp64", [False, True], ids=["float_params", "fp64_params"])
def test_reference_driver_compiles_links_and_runs_unchanged(tmp_path, facade_objects, fp64):
    exe, undefined = build_reference_driver(tmp_path, facade_objects, fp64)
    ctor = [ln for ln in undefined.splitlines() if "Grid::Grid(" in ln and "Basis*" in ln]
    assert ctor, undefined
    want = "double*, double*, Basis*, double, double, double, double" if fp64 else \
        "float*, float*, Basis*, float, float, float, float"
    assert any(want in ln for ln in ctor), ctor
    assert any("Grid::RK33(double" in ln for ln in undefined.splitlines())
    # wrong argument count: the reference's ERRCODE_INVALID_ARGUMENT
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1, (r.stdout, r.stderr)
    assert "Not enough command line arguments" in r.stderr
    # unreadable parameter file: ERRCODE_CANNOT_READ, after the output folder
    # and its log were created (cppsrc/driver.cpp:112-127, 190-195)
    r = subprocess.run([exe, "missing_params.txt", "out"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 3, (r.stdout, r.stderr)
    assert "Unable to open parameter file missing_params.txt" in r.stderr
    assert (tmp_path / "out" / "raw").is_dir() and (tmp_path / "out" / "_log.txt").exists()
