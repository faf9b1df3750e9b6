"""The snapshot files read by h5py, an independent HDF5 implementation (the
reader of the reference's plotting script, plotting.py:99-148).  Skipped where
h5py is not installed; neither the development container nor the GPU machines
of this project have it, so these tests document the check rather than run in
the standard suites."""
import os

import numpy as np
import pytest

from conftest import dg, workloads

h5py = pytest.importorskip("h5py")


def test_writer_file_read_by_h5py(tmp_path):
    a = np.random.default_rng(0).standard_normal((3, 4, 5, 6))
    p = str(tmp_path / "vel_0_3.h5")
    dg().hdf5_write(p, "velocity", a, 1.5)
    with h5py.File(p, "r") as f:
        assert set(f.keys()) == {"velocity", "time"}
        assert np.array_equal(f["velocity"][()], a)
        assert float(np.asarray(f["time"][()]).reshape(-1)[0]) == 1.5


@pytest.mark.gpu
def test_snapshot_files_read_by_h5py(tmp_path):
    """dg_write_snapshot's dRho, vel and coords files against dg_get_state /
    dg_get_grid, across two blocks."""
    cfg = workloads().gaussian_pulse(seed=0, num_elements=(2, 3, 2), order=3, width=1.25, sponge=1)
    cfg["NUM_BLOCKS"] = [2, 1, 1]
    cfg["DT"] = workloads().cfl_dt(cfg)
    with dg().Solver(cfg) as s:
        s.step(cfg["DT"], 2)
        rho, vel = s.state()
        coords, _ = s.grid()
        s.write_snapshot(str(tmp_path), 2, grid=True)
        t = s.time
    X = 2 * 4  # a block's x extent: 2 elements of K = 4 nodes
    for b in range(2):
        sl = slice(b * X, (b + 1) * X)
        with h5py.File(os.path.join(tmp_path, "raw", "dRho_%d_2.h5" % b), "r") as f:
            assert np.array_equal(f["rho"][()], rho[sl])
            assert float(np.asarray(f["time"][()]).reshape(-1)[0]) == t
        with h5py.File(os.path.join(tmp_path, "raw", "vel_%d_2.h5" % b), "r") as f:
            assert np.array_equal(f["velocity"][()], vel[:, sl])
        with h5py.File(os.path.join(tmp_path, "raw", "coords_%d_2.h5" % b), "r") as f:
            assert np.array_equal(f["coords"][()], coords[:, sl])
