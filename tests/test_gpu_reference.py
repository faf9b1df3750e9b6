"""GPU FP64 path against the reference's own solver: the golden vectors of
tests/golden (FP64-promoted reference build on identical seeded inputs), at
the stated step counts, through the C ABI and through the dg3d driver."""
import importlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, dg, max_rel, pressure

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")
with open(os.path.join(GOLDEN, "cases.json")) as f:
    CASES = json.load(f)
TOL = 1e-10


def golden_solver(cfg):
    return dg().Solver(cfg, os.path.join(GOLDEN, "matrices.txt"), os.path.join(GOLDEN, "hardcoded_coeff.txt"))


@pytest.mark.parametrize("name", sorted(CASES))
def test_matches_reference_golden(name):
    case = CASES[name]
    cfg = case["cfg"]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    with golden_solver(cfg) as s:
        s.step(case["dt"], case["steps"])
        rho, vel = s.state()
        t = s.time
    ep = max_rel(pressure(cfg, rho), pressure(cfg, g["rho"]))
    ev = max_rel(vel, g["vel"])
    assert ep <= TOL and ev <= TOL, (ep, ev)
    assert abs(t - float(g["time"])) <= 1e-13 * max(1.0, t)


def test_driver_end_to_end_matches_reference(tmp_path):
    """bin/dg3d on the reference-format parameter file of golden case c1_20,
    in a directory holding the same basis files the reference read; its HDF5
    snapshot must match the reference's output."""
    h5 = importlib.import_module("3ddg_gb300.h5read")
    exe = os.path.join(ROOT, "3ddg_gb300", "bin", "dg3d")
    for f in ("hardcoded_coeff.txt", "hardcoded_coeff2.txt", "matrices.txt"):
        shutil.copy(os.path.join(GOLDEN, f), tmp_path)
    shutil.copy(os.path.join(GOLDEN, "c1_20.params.txt"), tmp_path / "params.txt")
    r = subprocess.run([exe, "params.txt", "out"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Timestepping" in r.stdout and "Max dRho=" in r.stdout
    log = (tmp_path / "out" / "_log.txt").read_text()
    assert log.startswith("Parameters used:\n{\n")
    d = h5.read(str(tmp_path / "out" / "raw" / "dRho_0_20.h5"))
    v = h5.read(str(tmp_path / "out" / "raw" / "vel_0_20.h5"))
    g = np.load(os.path.join(GOLDEN, "c1_20.npz"))
    cfg = CASES["c1_20"]["cfg"]
    assert max_rel(pressure(cfg, d["rho"]), pressure(cfg, g["rho"])) <= TOL
    assert max_rel(v["velocity"], g["vel"]) <= TOL
    assert abs(float(d["time"][0]) - float(g["time"])) <= 1e-13
    c = h5.read(str(tmp_path / "out" / "raw" / "coords_0_0.h5"))
    assert c["coords"].shape == (3, 32, 32, 32)
    assert np.isclose(c["coords"][0, 0, 0, 0], -5.0) and np.isclose(c["coords"][2, -1, -1, -1], 5.0)
    ic = h5.read(str(tmp_path / "out" / "raw" / "dRho_0_0.h5"))
    assert ic["rho"].max() > 0.4


def test_driver_multiblock_writes_one_file_per_block(tmp_path):
    """NUM_BLOCKS = 2 1 2: one snapshot file pair per block (like one MPI rank
    each), together equal to the single-block run."""
    h5 = importlib.import_module("3ddg_gb300.h5read")
    exe = os.path.join(ROOT, "3ddg_gb300", "bin", "dg3d")
    W = importlib.import_module("3ddg_gb300.workloads")
    import refinputs
    cfg = W.gaussian_pulse(seed=0, num_elements=(2, 4, 2), order=2, width=1.25, sponge=1)
    cfg["NUM_BLOCKS"] = [2, 1, 2]
    cfg["DT"] = W.cfl_dt(cfg)
    p = dict(cfg)
    p.update(NUM_TIME_SUBSTEPS=3, NUM_OUTSTEPS=2, FREQ_TERMINAL=1, BOOL_FILE=1)
    refinputs.write_params(str(tmp_path / "params.txt"), p)
    r = subprocess.run([exe, "params.txt", "out"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    parts = {b: h5.read(str(tmp_path / "out" / "raw" / ("dRho_%d_6.h5" % b)))["rho"] for b in range(4)}
    assert all(a.shape == (6, 12, 6) for a in parts.values())
    full = np.zeros((12, 12, 12))
    for b, a in parts.items():
        bx, bz = b // 2, b % 2
        full[bx * 6:(bx + 1) * 6, :, bz * 6:(bz + 1) * 6] = a
    single = dict(cfg)
    single["NUM_BLOCKS"] = [1, 1, 1]
    single["NUM_ELEMENTS"] = [4, 4, 4]
    with dg().Solver(single) as s:
        s.step(cfg["DT"], 6)
        rho, _ = s.state()
    assert max_rel(full, rho) <= 1e-12
