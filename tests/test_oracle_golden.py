"""The C oracle against golden vectors from the reference's own solver
(tests/golden/*.npz, produced by tests/golden/make_golden.py with the
FP64-promoted reference build).  CPU only."""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, max_rel, pressure

GOLDEN = os.path.join(ROOT, "tests", "golden")
with open(os.path.join(GOLDEN, "cases.json")) as f:
    CASES = json.load(f)

FAST = [n for n in CASES if not n.startswith("c1_200")]


def run_oracle(name):
    import pyoracle
    import refinputs
    case = CASES[name]
    cfg = case["cfg"]
    order = int(cfg["ORDER"])
    M, S = refinputs.read_matrices(os.path.join(GOLDEN, "matrices.txt"), order)
    z = refinputs.read_zeros(os.path.join(GOLDEN, "hardcoded_coeff.txt"), order)
    o = pyoracle.Oracle(cfg, M, S, z)
    o.run(case["dt"], case["steps"])
    return cfg, o


@pytest.mark.parametrize("name", FAST)
def test_oracle_matches_reference(name):
    cfg, o = run_oracle(name)
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    rho, vel = o.state()
    assert rho.shape == g["rho"].shape
    assert max_rel(pressure(cfg, rho), pressure(cfg, g["rho"])) <= 1e-12
    assert max_rel(vel, g["vel"]) <= 1e-12
    assert abs(o.time - float(g["time"])) <= 1e-14 * max(1.0, abs(float(g["time"])))


def test_oracle_matches_reference_config1_200_steps():
    """Config 1 at its stated step count (200)."""
    cfg, o = run_oracle("c1_200")
    g = np.load(os.path.join(GOLDEN, "c1_200.npz"))
    rho, vel = o.state()
    assert max_rel(pressure(cfg, rho), pressure(cfg, g["rho"])) <= 1e-11
    assert max_rel(vel, g["vel"]) <= 1e-11


def test_reference_fp32_build_is_close_to_fp64():
    """Sanity cross-check recorded with the fixture: the reference as shipped
    (float state, double line solves) stays within FP32 rounding of ref64."""
    g = np.load(os.path.join(GOLDEN, "c1_20.npz"))
    assert max_rel(g["rho32"], g["rho"]) < 1e-5


def test_golden_inputs_are_reproducible(tmp_path):
    """The committed basis files are what oracle/refinputs.py generates."""
    import refinputs
    refinputs.write_coeff_files(str(tmp_path))
    refinputs.write_matrices(str(tmp_path))
    for f in ("hardcoded_coeff.txt", "matrices.txt"):
        a = open(os.path.join(GOLDEN, f)).read().split()
        b = open(os.path.join(tmp_path, f)).read().split()
        assert len(a) == len(b)
        # identical up to the last bit of a few Newton-iterated nodes
        nd = sum(1 for x, y in zip(a, b) if x != y)
        assert nd <= len(a) // 50, nd


def total_mass_after(rk_exact, steps=5):
    import pyoracle
    import refinputs
    cfg = dict(CASES["n4_linear_nodiff"]["cfg"])
    cfg["BC_IS_PERIODIC"] = [1, 1, 1]
    cfg["RK_EXACT"] = rk_exact
    order = int(cfg["ORDER"])
    M, S = refinputs.read_matrices(os.path.join(GOLDEN, "matrices.txt"), order)
    z = refinputs.read_zeros(os.path.join(GOLDEN, "hardcoded_coeff.txt"), order)
    o = pyoracle.Oracle(cfg, M, S, z)
    w1 = M.sum(axis=1)  # integral of each basis function on [0, 1]
    ne = cfg["NUM_ELEMENTS"]
    wt = np.tile(w1, ne[0])[:, None, None] * np.tile(w1, ne[1])[None, :, None] * np.tile(w1, ne[2])[None, None, :]
    r0, _ = o.state()
    o.run(CASES["n4_linear_nodiff"]["dt"], steps)
    r1, _ = o.state()
    return float((wt * r0).sum()), float((wt * r1).sum())


def test_oracle_conserves_mass_periodic_linear():
    """Periodic, linear, no sponge/diffusion, exact RK weights: the DG scheme
    conserves total mass sum(w drho) to rounding (size-independent)."""
    m0, m1 = total_mass_after(rk_exact=1)
    assert abs(m1 - m0) <= 1e-13 * abs(m0)


def test_reference_rk_weights_scale_total_mass():
    """With the reference's stage-3 weights (float literals 2.0F/3.0F and
    1.0F/3.0F, cppsrc/Grid.cpp:826-827, kept float-rounded by its FP64 build)
    the weights sum to 1 + 2.98e-8, so total mass grows by exactly that factor
    per step."""
    m0, m1 = total_mass_after(rk_exact=0)
    g = float(np.float32(2.0) / np.float32(3.0)) + float(np.float32(1.0) / np.float32(3.0))
    assert abs(m1 / m0 - g ** 5) <= 1e-13
