"""The seeded synthetic workloads (3ddg_gb300/workloads.py) against the
configurations they stand for: the 64^3-element FP64 case, the batched
distribution, the CFL time step, and the focal-axis harmonic measure.  CPU
only."""
import math

import numpy as np
import pytest

from conftest import workloads


def test_cfl_dt_formula():
    W = workloads()
    cfg = dict(ORDER=4, ELEMENT_WIDTH=[0.5, 0.25, 1.0], C0=1.5)
    assert math.isclose(W.cfl_dt(cfg), 0.5 / (9 * 1.5 * (2.0 + 4.0 + 1.0)), rel_tol=1e-15)
    assert math.isclose(W.cfl_dt(cfg, cfl=0.25), 0.5 * W.cfl_dt(cfg), rel_tol=1e-15)


def test_config1_and_config3():
    W = workloads()
    c1, c3 = W.config1(seed=0), W.config3(seed=0)
    assert c1["ORDER"] == 3 and c1["NUM_ELEMENTS"] == [8, 8, 8] and c1["STEPS"] == 200
    # a 1 cm cube centred on the origin, 2-element sponges, water
    assert np.allclose(np.array(c1["NUM_ELEMENTS"]) * c1["ELEMENT_WIDTH"], 10.0)
    assert c1["STARTING_CORNER"] == [-5.0, -5.0, -5.0] and c1["BC_SPONGE_WIDTH"] == [2] * 6
    assert (c1["C0"], c1["RHO0"], c1["B_OVER_A"]) == (1.5, 1000.0, 5.0)
    # 1 MPa pulse amplitude (drho = p / c0^2) with +/-1e-3 seeded jitter
    assert abs(c1["IC_DRHO_AMPLITUDE"] * 1.5 ** 2 - 1.0) <= 1e-3
    assert W.config1(seed=1)["IC_DRHO_AMPLITUDE"] != c1["IC_DRHO_AMPLITUDE"]
    assert c3.get("PRECISION") == 32 and {k: v for k, v in c3.items() if k != "PRECISION"} == c1


def test_config2_is_the_64_cubed_tone_burst_case():
    W = workloads()
    c = W.config2(seed=0)
    ne = [e * b for e, b in zip(c["NUM_ELEMENTS"], c["NUM_BLOCKS"])]
    assert ne == [64, 64, 64] and c["NUM_BLOCKS"] == [2, 2, 2] and c["ORDER"] == 4
    assert W.dof_count(c) == 4 * 64 ** 3 * 125  # 32.8 M nodes
    assert c["SRC_FACE"] == 4 and c["BC_SPONGE_WIDTH"] == [3, 3, 3, 3, 0, 3]
    assert (c["SRC_AMPLITUDE"], c["SRC_FREQUENCY"], c["SRC_CYCLES"]) == (2.0, 1.0, 5.0)
    # seeded phase offset of at most 0.5 % of a cycle, different per seed
    assert abs(c["SRC_PHASE"]) <= 2 * math.pi * 0.005
    assert W.config2(seed=3)["SRC_PHASE"] != c["SRC_PHASE"]
    assert c["STEPS"] == 1000 and math.isclose(c["DT"], W.cfl_dt(c), rel_tol=1e-15)


def test_config4_distribution():
    W = workloads()
    cfgs = W.config4(seed=0)
    assert len(cfgs) == 256
    assert cfgs == W.config4(seed=0)  # seeded
    ne = np.array([c["NUM_ELEMENTS"] for c in cfgs])
    assert ne.min() >= 4 and ne.max() <= 24 and len(np.unique(ne)) > 15
    orders = {c["ORDER"] for c in cfgs}
    assert orders == {2, 3, 4, 5}
    amp = np.array([c["SRC_AMPLITUDE"] for c in cfgs])
    assert amp.min() >= 0.1 and amp.max() <= 5.0
    # log-uniform: the median sits near the geometric mean of the range
    assert 0.4 < np.median(amp) < 1.6
    freq = np.array([c["SRC_FREQUENCY"] for c in cfgs])
    assert freq.min() >= 0.5 and freq.max() <= 2.0
    sponge = np.array([c["BC_SPONGE_WIDTH"][0] for c in cfgs])
    assert set(sponge.tolist()) <= {2, 3, 4} and len(set(sponge.tolist())) == 3
    c0 = np.array([c["C0"] for c in cfgs])
    assert c0.min() >= 1.45 and c0.max() <= 1.60
    for c in cfgs:
        assert c["PRECISION"] == 32 and c["STEPS"] == 500 and c["SRC_FACE"] == 4
        assert c["BC_SPONGE_WIDTH"][4] == 0 and math.isclose(c["DT"], W.cfl_dt(c), rel_tol=1e-15)


@pytest.mark.parametrize("f1", [0.25, 0.5])
def test_harmonics_recovers_a_known_signal(f1):
    """The measure the FP32 form's 2nd-harmonic error is stated with: a
    fundamental and its second harmonic on exact DFT bins come back with
    their frequency and amplitudes."""
    W = workloads()
    n, dt = 4096, 1.0 / 64
    t = np.arange(n) * dt
    p = 0.8 * np.sin(2 * np.pi * f1 * t) + 0.05 * np.sin(2 * np.pi * 2 * f1 * t + 0.3)
    f, a1, a2 = W.harmonics(t, p)
    assert math.isclose(f, f1, rel_tol=1e-12)
    assert abs(a1 - 0.8) <= 0.8 * 1e-3 and abs(a2 - 0.05) <= 0.05 * 1e-2
