"""The library-free HDF5 reader (dg_hdf5_read, the counterpart of the
reference's hdf5input, cppsrc/HDF5Functions.cpp:398-463) and the host
hdf5input mirror: round trips through the writer, the reader's other
datatype paths (files patched byte-wise), and the reference's error codes
-1 file, -2 dataset, -3 dataspace, -4 datatype.  CPU only."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, dg

F64_TYPE = bytes([0x11, 0x20, 63, 0, 8, 0, 0, 0])  # datatype message head of the writer's float64


def write(tmp_path, name, arr, t=0.5, fname="a.h5"):
    p = str(tmp_path / fname)
    dg().hdf5_write(p, name, arr, t)
    return p


def patch(path, old, new, count=1):
    raw = open(path, "rb").read()
    assert raw.count(old) >= count
    raw = raw.replace(old, new, count)
    open(path, "wb").write(raw)


def code_of(fn):
    m = dg()
    with pytest.raises(m.DGError) as e:
        fn()
    return e.value.code


@pytest.mark.parametrize("shape", [(1,), (7,), (3, 5), (4, 3, 6), (3, 2, 4, 5), (2, 1, 3, 1, 2)])
def test_roundtrip_exact(tmp_path, shape):
    m = dg()
    a = np.random.default_rng(len(shape)).standard_normal(shape) * 1e3
    p = write(tmp_path, "velocity", a, 3.25)
    b, cls = m.hdf5_read(p, "velocity")
    assert cls == 1 and b.shape == a.shape and np.array_equal(a, b)
    t, _ = m.hdf5_read(p, "time")
    assert t.tolist() == [3.25]


def test_special_values_roundtrip(tmp_path):
    m = dg()
    a = np.array([0.0, -0.0, np.inf, -np.inf, 5e-324, 1.7976931348623157e308, np.nan])
    b, _ = m.hdf5_read(write(tmp_path, "rho", a), "rho")
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_signed_integer_dataset(tmp_path):
    """Datatype patched to a signed 64-bit integer: the stored bytes read as int64."""
    m = dg()
    ints = np.array([[-3, 7, 0], [2**40, -(2**40), 1]], dtype=np.int64)
    p = write(tmp_path, "rho", ints.view(np.float64))
    patch(p, F64_TYPE, bytes([0x10, 0x08, 0, 0, 8, 0, 0, 0]))
    b, cls = m.hdf5_read(p, "rho")
    assert cls == 0 and np.array_equal(b, ints.astype(np.float64))


def test_big_endian_float_dataset(tmp_path):
    m = dg()
    a = np.random.default_rng(5).standard_normal((4, 3))
    p = write(tmp_path, "rho", a.byteswap())
    patch(p, F64_TYPE, bytes([0x11, 0x21, 63, 0, 8, 0, 0, 0]))
    b, _ = m.hdf5_read(p, "rho")
    assert np.array_equal(a, b)


def test_missing_file_is_file_error(tmp_path):
    m = dg()
    assert code_of(lambda: m.hdf5_read(str(tmp_path / "none.h5"), "rho")) == -1


def test_not_hdf5_is_file_error(tmp_path):
    m = dg()
    p = tmp_path / "x.h5"
    p.write_bytes(b"not an hdf5 file at all" * 40)
    assert code_of(lambda: m.hdf5_read(str(p), "rho")) == -1


def test_missing_dataset_is_dataset_error(tmp_path):
    m = dg()
    p = write(tmp_path, "rho", np.zeros((2, 2, 2)))
    assert code_of(lambda: m.hdf5_read(p, "velocity")) == -2


def test_chunked_layout_is_dataset_error(tmp_path):
    m = dg()
    a = np.arange(24.0).reshape(2, 3, 4)
    p = write(tmp_path, "rho", a)
    # layout message of the first dataset ("rho" sorts before "time"): version 3, class 1 -> 2
    raw = open(p, "rb").read()
    head = bytes([0x08, 0x00, 0x18, 0x00, 0, 0, 0, 0, 3, 1])
    assert raw.count(head) == 2
    patch(p, head, head[:-1] + bytes([2]))
    assert code_of(lambda: m.hdf5_read(p, "rho")) == -2
    t, _ = m.hdf5_read(p, "time")  # the other dataset is untouched
    assert t.tolist() == [0.5]


def test_truncated_data_is_dataspace_error(tmp_path):
    m = dg()
    p = write(tmp_path, "rho", np.ones((40, 40)), fname="t.h5")
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:-1000])
    assert code_of(lambda: m.hdf5_read(p, "time")) == -3


def test_string_datatype_is_datatype_error(tmp_path):
    m = dg()
    p = write(tmp_path, "rho", np.ones((3, 3)))
    patch(p, F64_TYPE, bytes([0x13, 0x00, 0, 0, 8, 0, 0, 0]))
    assert code_of(lambda: m.hdf5_read(p, "rho")) == -4


def test_small_capacity_is_rejected(tmp_path):
    import ctypes as C
    m = dg()
    p = write(tmp_path, "rho", np.ones(10))
    out = np.empty(9)
    rc = m.lib().dg_hdf5_read(p.encode(), b"rho", 0, None, None, out.ctypes.data_as(C.c_void_p), 9, None)
    assert rc == -3 and b"more than" in m.lib().dg_last_error()


HARNESS = r'''
#include <cstdio>
#include <string>
#include <vector>
#include "HDF5Functions.h"
int main(int argc, char** argv)
{
    int X = std::stoi(argv[3]), Y = std::stoi(argv[4]), Z = std::stoi(argv[5]);
    std::vector<std::vector<std::vector<double>>> d(X, std::vector<std::vector<double>>(Y, std::vector<double>(Z, -1.0)));
    int rc = hdf5input(d, argv[1], argv[2], X, Y, Z);
    std::printf("rc=%d\n", rc);
    if (rc == 0)
        for (int x = 0; x < X; x++)
            for (int y = 0; y < Y; y++)
                for (int z = 0; z < Z; z++) std::printf("%.17g\n", d[x][y][z]);
    return 0;
}
'''


@pytest.fixture(scope="module")
def hdf5input_bin(tmp_path_factory):
    m = dg()
    m.lib()
    d = tmp_path_factory.mktemp("harness")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    host = os.path.join(ROOT, "3ddg_gb300", "csrc", "host")
    exe = d / "h"
    cmd = ["g++", "-std=c++17", "-O1", "-I" + host, "-I" + os.path.join(ROOT, "include"), str(src),
           os.path.join(host, "HDF5Functions.cpp"), os.path.join(host, "Grid.cpp"), os.path.join(host, "Basis.cpp"),
           "-L" + os.path.dirname(m.LIB_PATH), "-ldg3d", "-Wl,-rpath," + os.path.dirname(m.LIB_PATH),
           "-lpthread", "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True)
    return str(exe)


def test_hdf5input_index_mapping(tmp_path, hdf5input_bin):
    """hdf5input reads a [Z][Y][X] dataset into data3D[x][y][z] and prints the
    datatype class (1 = floating point) first."""
    X, Y, Z = 3, 4, 5
    stored = np.random.default_rng(2).standard_normal((Z, Y, X))
    p = write(tmp_path, "rho", stored)
    out = subprocess.run([hdf5input_bin, p, "rho", str(X), str(Y), str(Z)], capture_output=True, text=True).stdout
    lines = out.split()
    assert lines[0] == "1" and lines[1] == "rc=0"
    got = np.array([float(v) for v in lines[2:]]).reshape(X, Y, Z)
    assert np.array_equal(got, stored.transpose(2, 1, 0))


@pytest.mark.parametrize("case,code,msg", [("nofile", -1, "FileIException"), ("noset", -2, "DataSetIException"),
                                           ("size", -3, "DataSpaceIException")])
def test_hdf5input_error_codes(tmp_path, hdf5input_bin, case, code, msg):
    p = write(tmp_path, "rho", np.zeros((2, 2, 2)))
    path, name, dims = p, "rho", ("2", "2", "2")
    if case == "nofile":
        path = str(tmp_path / "missing.h5")
    elif case == "noset":
        name = "velocity"
    else:
        dims = ("2", "2", "3")
    out = subprocess.run([hdf5input_bin, path, name, *dims], capture_output=True, text=True).stdout
    assert msg in out and ("rc=%d" % code) in out


def scipy_matlab_data():
    """scipy's MATLAB test data: testhdf5_7.4_GLNX86.mat is an HDF5 file
    written by the HDF5 library (MATLAB's, with a 512-byte user block and a
    version-2 data layout message) holding the 1 x 9 double "testdouble";
    testdouble_7.1_GLNX86.mat holds the same variable in MATLAB's own v5
    format, which scipy.io.loadmat decodes without any HDF5 code."""
    sio = pytest.importorskip("scipy.io")
    d = os.path.join(os.path.dirname(sio.matlab.__file__), "tests", "data")
    h5, v5 = os.path.join(d, "testhdf5_7.4_GLNX86.mat"), os.path.join(d, "testdouble_7.1_GLNX86.mat")
    if not (os.path.exists(h5) and os.path.exists(v5)):
        pytest.skip("scipy's MATLAB test data is not installed")
    return h5, sio.loadmat(v5)["testdouble"]


def test_readers_read_a_file_written_by_the_hdf5_library():
    """Both readers (dg_hdf5_read and the Python h5read) on a file that the
    HDF5 library wrote, against an independent decoder of the same values."""
    import importlib
    h5path, want = scipy_matlab_data()
    m = dg()
    a, cls = m.hdf5_read(h5path, "testdouble")
    assert cls == 1 and a.shape == (9, 1)  # MATLAB stores the 1 x 9 array column-major
    assert np.array_equal(a.T, want)
    b = importlib.import_module("3ddg_gb300.h5read").read(h5path)["testdouble"]
    assert np.array_equal(b, a)
