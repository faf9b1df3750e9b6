"""Batched form (dg_batch_*): uneven FP32 problems in one persistent kernel per
RK stage.  Checked against the single-problem FP32 path and the FP64 oracle,
and for independence from the batch-mates (bitwise)."""
import numpy as np
import pytest

from conftest import dg, max_rel, pressure, workloads

pytestmark = pytest.mark.gpu


def mixed(n=6, seed=3):
    W = workloads()
    cfgs = W.config4(seed=seed, n=n, steps=40)
    for c in cfgs:  # keep the test quick
        c["NUM_ELEMENTS"] = [min(v, 8) for v in c["NUM_ELEMENTS"]]
        c["STARTING_CORNER"] = [-0.5 * c["NUM_ELEMENTS"][0] * 0.25, -0.5 * c["NUM_ELEMENTS"][1] * 0.25, 0.0]
    return cfgs


def test_batch_matches_single_problem_fp32():
    m = dg()
    cfgs = mixed()
    assert len({c["ORDER"] for c in cfgs}) >= 3
    with m.Batch(cfgs) as b:
        b.step(40)
        got = [b.state(i) for i in range(len(cfgs))]
        for i in range(len(cfgs)):
            assert b.info(i)[1] == 40
    for c, (r, v) in zip(cfgs, got):
        with m.Solver(c) as s:
            s.step(c["DT"], 40)
            r1, v1 = s.state()
        assert np.max(np.abs(r1)) > 0  # the burst entered the domain
        assert max_rel(pressure(c, r), pressure(c, r1)) <= 2e-5
        assert max_rel(v, v1) <= 2e-5


def test_batch_anisotropic_elements_match_single_problem_fp32():
    """Different element widths per axis in every problem: the batch applies
    each axis's 1/w after the line sums with axis-free operator rows."""
    m = dg()
    W = workloads()
    cfgs = mixed(n=4, seed=5)
    for k, c in enumerate(cfgs):
        c["ELEMENT_WIDTH"] = [0.25, 0.2 + 0.02 * k, 0.3]
        c["STARTING_CORNER"] = [-0.5 * c["NUM_ELEMENTS"][a] * c["ELEMENT_WIDTH"][a] for a in range(2)] + [0.0]
        c["DT"] = W.cfl_dt(c)
    with m.Batch(cfgs) as b:
        b.step(30)
        got = [b.state(i) for i in range(len(cfgs))]
    for c, (r, v) in zip(cfgs, got):
        with m.Solver(c) as s:
            s.step(c["DT"], 30)
            r1, v1 = s.state()
        assert np.max(np.abs(r1)) > 0
        assert max_rel(pressure(c, r), pressure(c, r1)) <= 2e-5
        assert max_rel(v, v1) <= 2e-5


def test_batch_result_independent_of_batch_mates():
    m = dg()
    cfgs = mixed(n=5, seed=7)
    with m.Batch(cfgs) as b:
        b.step(25)
        mix = b.state(2)
    with m.Batch([cfgs[2]]) as b1:
        b1.step(25)
        alone = b1.state(0)
    assert np.array_equal(mix[0], alone[0]) and np.array_equal(mix[1], alone[1])


def test_batch_stops_each_problem_after_its_steps():
    m = dg()
    cfgs = mixed(n=3, seed=11)
    cfgs[0]["STEPS"], cfgs[1]["STEPS"], cfgs[2]["STEPS"] = 5, 12, 30
    with m.Batch(cfgs) as b:
        b.step(20)
        done = [b.info(i)[1] for i in range(3)]
        r0 = b.state(0)[0]
        b.step(5)
        assert np.array_equal(b.state(0)[0], r0)
    assert done == [5, 12, 20]


def test_batch_against_fp64_oracle(oracle_for):
    """One batched problem against the FP64 oracle: relative L2 pressure
    error within the FP32 bound of the precision form."""
    m = dg()
    c = mixed(n=1, seed=5)[0]
    c64 = dict(c)
    c64.pop("PRECISION")
    o = oracle_for(c64)
    with m.Batch([c]) as b:
        b.step(30)
        r, _ = b.state(0)
    o.run(c["DT"], 30)
    ro, _ = o.state()
    p, po = pressure(c, r), pressure(c, ro)
    assert np.linalg.norm(p - po) / np.linalg.norm(po) <= 1e-5


def test_autotune_keeps_results():
    m = dg()
    cfgs = mixed(n=4, seed=9)
    with m.Batch(cfgs) as b:
        b.step(3)
        rep = b.autotune(2)
        assert "ctas_per_sm" in rep
        b.step(7)
        tuned = b.state(1)
    with m.Batch(cfgs) as b2:
        b2.step(10)
        ref = b2.state(1)
    assert np.array_equal(tuned[0], ref[0])


def test_batch_tiny_and_ragged_problems():
    """Problems of 1 to 6 elements at every order the batch takes, all in one
    batch: tiles shorter than a pass (EPB up to 8 elements), every face on the
    boundary, the source face on each.  Each matches the single-problem FP32
    path within the FP32 tolerance of the other batch tests."""
    m = dg()
    W = workloads()
    base = W.config4(seed=13, n=1, steps=20)[0]
    cfgs = []
    for order in (1, 2, 3, 4, 5):
        for ne in ((1, 1, 1), (1, 2, 3), (3, 1, 2)):
            c = dict(base)
            c["ORDER"] = order
            c["NUM_ELEMENTS"] = list(ne)
            c["BC_SPONGE_WIDTH"] = [1, 1, 1, 1, 0, 1]
            c["STARTING_CORNER"] = [-0.5 * ne[0] * 0.25, -0.5 * ne[1] * 0.25, 0.0]
            c["DT"] = W.cfl_dt(c)
            c["STEPS"] = 20
            cfgs.append(c)
    with m.Batch(cfgs) as b:
        b.step(20)
        got = [b.state(i) for i in range(len(cfgs))]
    for c, (r, v) in zip(cfgs, got):
        with m.Solver(c) as s:
            s.step(c["DT"], 20)
            r1, v1 = s.state()
        assert np.max(np.abs(r1)) > 0
        assert max_rel(pressure(c, r), pressure(c, r1)) <= 2e-5, (c["ORDER"], c["NUM_ELEMENTS"])
        assert max_rel(v, v1) <= 2e-5, (c["ORDER"], c["NUM_ELEMENTS"])
