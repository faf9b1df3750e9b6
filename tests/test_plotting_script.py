"""The reference's plotting.py (the reader of the snapshot files) run on a
snapshot set that this package's driver wrote: tests/golden/plotting_n3_b211/,
made by tests/golden/make_plotting_fixture.py with bin/dg3d on a two-block,
order-3 run (NUM_BLOCKS = 2 1 1, snapshots at time steps 0, 2, 4).

plotting.py reads ``results/_log.txt`` for the block and element counts, then
every block's ``raw/{coords,ba,diff,rho0,c0}_<rank>_0.h5`` and, for every time
step, ``raw/dRho_<rank>_<ts>.h5`` / ``raw/vel_<rank>_<ts>.h5``, and assembles
the blocks by rank (plotting.py:30-158).  Neither h5py nor matplotlib is
installed here, so the script runs with matplotlib replaced by mocks and
h5py by a module over this package's HDF5 reader (3ddg_gb300/h5read.py, which
is itself checked against a file the HDF5 library wrote,
tests/test_hdf5_read.py).  What this checks is the file and dataset naming,
the shapes, the rank numbering and the log format that plotting.py depends
on; the byte-level HDF5 encoding is checked by the reader tests.  The
reference's plotting.py is copied into a temporary directory at test time
(never committed); the test is skipped where the reference sources are absent.
CPU only."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

FIXTURE = os.path.join(ROOT, "tests", "golden", "plotting_n3_b211")


def reference_plotting():
    d = os.environ.get("DG3D_REFERENCE_SRC")
    if not d:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"], capture_output=True,
                           text=True)
        d = r.stdout.strip()
    return os.path.join(os.path.dirname(d.rstrip("/")), "plotting.py") if d else ""


PLOTTING = reference_plotting()
pytestmark = pytest.mark.skipif(not (PLOTTING and os.path.isfile(PLOTTING)), reason="reference sources not present")

RUNNER = r'''
import importlib, os, runpy, sys
from unittest import mock
sys.path.insert(0, sys.argv[1])
h5read = importlib.import_module("3ddg_gb300.h5read")


class File:
    """The part of h5py.File that plotting.py uses: open for reading,
    index a dataset by name, use as a context manager."""

    def __init__(self, path, mode="r"):
        assert mode == "r"
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self._d = h5read.read(path)

    def __getitem__(self, name):
        return self._d[name]

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


h5py = type(sys)("h5py")
h5py.File = File
sys.modules["h5py"] = h5py
for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.cm", "matplotlib.ticker", "mpl_toolkits",
             "mpl_toolkits.mplot3d", "mpl_toolkits.mplot3d.axes3d"):
    sys.modules[name] = mock.MagicMock()
g = runpy.run_path("plotting.py", run_name="__main__")
import numpy as np
np.save("assembled_drho.npy", g["dRhoVals"])
np.save("assembled_x.npy", g["xVals"])
'''


def test_reference_plotting_reads_driver_snapshots(tmp_path):
    h5 = __import__("importlib").import_module("3ddg_gb300.h5read")
    shutil.copytree(FIXTURE, tmp_path / "results")
    shutil.copy(PLOTTING, tmp_path / "plotting.py")
    (tmp_path / "runner.py").write_text(RUNNER)
    r = subprocess.run([sys.executable, "runner.py", ROOT], cwd=tmp_path, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    out = r.stdout
    # the log's block and element counts (plotting.py:33-46)
    assert "Param file read, B= [2, 1, 1] , E= [2, 2, 2]" in out, out[:500]
    # every snapshot time step was read for both ranks (a failed read skips
    # the step silently, plotting.py:155-156)
    steps = [int(ln.split()[1]) for ln in out.splitlines() if ln.startswith("T= ")]
    assert steps == [0, 2, 4], out[-1000:]
    # the blocks assembled by rank are the blocks the driver wrote
    full = np.load(tmp_path / "assembled_drho.npy")
    assert full.shape == (16, 8, 8)
    for b in range(2):
        part = h5.read(os.path.join(FIXTURE, "raw", "dRho_%d_4.h5" % b))["rho"]
        assert np.array_equal(full[8 * b:8 * (b + 1)], part)
    x = np.load(tmp_path / "assembled_x.npy")
    assert np.isclose(x[0, 0, 0], -2.5) and np.isclose(x[-1, 0, 0], 2.5)
    assert np.all(np.diff(x[:, 0, 0]) >= 0)
