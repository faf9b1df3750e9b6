"""Restart from a snapshot (dg_read_snapshot; the reference's dormant reader
is hdf5input, cppsrc/HDF5Functions.cpp:398-463): an FP64 run that writes a
snapshot and continues equals, bit for bit, a fresh handle that reads the
snapshot and continues; across blocks and with the time-dependent tone-burst
source.  FP32 continues within its stated tolerance."""
import numpy as np
import pytest

from conftest import dg, workloads

pytestmark = pytest.mark.gpu


def small(ne=(4, 3, 5), blocks=(1, 1, 1)):
    W = workloads()
    cfg = W.gaussian_pulse(seed=4, num_elements=ne, order=3, width=1.25, sponge=1)
    cfg["NUM_BLOCKS"] = list(blocks)
    cfg["IC_VX_AMPLITUDE"] = 0.001
    cfg["DT"] = W.cfl_dt(cfg)
    return cfg


def burst():
    W = workloads()
    cfg = W.scaled(W.config2(seed=2), (3, 3, 4))
    cfg["ORDER"] = 3
    cfg["DT"] = W.cfl_dt(cfg)
    return cfg


def continue_vs_restart(cfg, solver_for, tmp_path, n1, n2):
    a = solver_for(cfg)
    a.step(cfg["DT"], n1)
    t1 = a.time
    a.write_snapshot(str(tmp_path), n1)
    a.step(cfg["DT"], n2)
    b = solver_for(cfg)
    b.read_snapshot(str(tmp_path), n1)
    assert b.time == t1
    b.step(cfg["DT"], n2)
    assert b.time == a.time
    return a.state(), b.state()


@pytest.mark.parametrize("blocks", [(1, 1, 1), (2, 1, 2)])
def test_fp64_restart_is_bit_identical(blocks, solver_for, tmp_path):
    cfg = small(ne=(4, 3, 4) if blocks == (1, 1, 1) else (2, 3, 2), blocks=blocks)
    (ra, va), (rb, vb) = continue_vs_restart(cfg, solver_for, tmp_path, 5, 4)
    assert np.array_equal(ra, rb) and np.array_equal(va, vb)


def test_fp64_restart_with_tone_burst(solver_for, tmp_path):
    cfg = burst()
    (ra, va), (rb, vb) = continue_vs_restart(cfg, solver_for, tmp_path, 30, 10)
    assert np.max(np.abs(ra)) > 0
    assert np.array_equal(ra, rb) and np.array_equal(va, vb)


def test_fp32_restart_within_tolerance(solver_for, tmp_path):
    cfg = small()
    cfg["PRECISION"] = 32
    (ra, va), (rb, vb) = continue_vs_restart(cfg, solver_for, tmp_path, 5, 5)
    assert np.linalg.norm(ra - rb) <= 1e-6 * np.linalg.norm(ra)


def test_restart_shape_mismatch_is_dataspace_error(solver_for, tmp_path):
    m = dg()
    cfg = small()
    a = solver_for(cfg)
    a.write_snapshot(str(tmp_path), 0)
    other = small(ne=(4, 3, 6))
    b = solver_for(other)
    with pytest.raises(m.DGError, match=r"\(-3\)"):
        b.read_snapshot(str(tmp_path), 0)
    with pytest.raises(m.DGError, match=r"\(-1\)"):
        b.read_snapshot(str(tmp_path), 7)
