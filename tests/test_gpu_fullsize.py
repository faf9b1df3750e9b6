"""Config 2 at its full size (64^3 elements at N = 4, 32.8 M nodes, 2x2x2
blocks), with a Gaussian pulse added to the tone burst so that every element
carries data: one RK step against the C oracle (about 30 s of one host core),
and size-independent properties over several steps: 2x2x2 blocks are bitwise
one block, total mass is conserved with periodic boundaries, the FP32 form
stays within its error bound.  Config 4 at its full size (256 problems): the
batched form agrees with the single-problem FP32 path."""
import numpy as np
import pytest

from conftest import dg, max_rel, pressure, workloads

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10


def config2_with_pulse(**kw):
    W = workloads()
    cfg = W.config2(seed=0)
    cfg.update(IC_X_GAUSS=1, IC_Y_GAUSS=1, IC_Z_GAUSS=1, IC_DRHO_AMPLITUDE=1.0 / cfg["C0"] ** 2,
               IC_SIGMA=0.5, IC_CENTER_X=0.5, IC_CENTER_Y=-0.25, IC_CENTER_Z=8.0, IC_VZ_AMPLITUDE=1e-4)
    cfg.update(kw)
    return cfg


def test_full_size_step_matches_oracle(solver_for, oracle_for):
    cfg = config2_with_pulse()
    s = solver_for(cfg)
    s.step(cfg["DT"], 1)
    r_g, v_g = s.state()
    s.close()
    o = oracle_for(cfg)
    o.run(cfg["DT"], 1)
    r_o, v_o = o.state()
    o.close()
    assert r_g.shape == (320, 320, 320)
    ep = max_rel(pressure(cfg, r_g), pressure(cfg, r_o))
    ev = max_rel(v_g, v_o)
    assert ep <= STEP_TOL and ev <= STEP_TOL, (ep, ev)


def test_full_size_blocks_bitwise_one_block(solver_for):
    c8 = config2_with_pulse()
    c1 = dict(c8, NUM_BLOCKS=[1, 1, 1], NUM_ELEMENTS=[64, 64, 64])
    out = []
    for c in (c8, c1):
        s = solver_for(c)
        s.step(c["DT"], 3)
        out.append(s.state())
        s.close()
    assert np.max(np.abs(out[0][0])) > 0
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("precision,tol", [(64, 1e-11), (32, 1e-6)])
def test_full_size_periodic_mass_conserved(precision, tol, solver_for):
    """With periodic boundaries, no sponge and no source the weighted sum of
    drho (its integral: the LGL weights are the column sums of M) changes only
    by rounding; exact RK weights (the reference's float weights scale it by
    1 + 2.98e-8 per step)."""
    cfg = config2_with_pulse(BC_IS_PERIODIC=[1, 1, 1], EVALUATE_SPONGE=0, SRC_FACE=-1, RK_EXACT=1,
                             PRECISION=precision)
    m = dg()
    w = m.line_operators(cfg["ORDER"])["mass"].sum(axis=0)
    s = solver_for(cfg)
    r0, _ = s.state()
    K = cfg["ORDER"] + 1
    wx = np.tile(w, r0.shape[0] // K)
    W3 = wx[:, None, None] * wx[None, :, None] * wx[None, None, :]
    m0, a0 = float(np.sum(W3 * r0)), float(np.sum(W3 * np.abs(r0)))
    s.step(cfg["DT"], 5)
    r5, v5 = s.state()
    s.close()
    assert np.max(np.abs(v5)) > 0
    assert abs(float(np.sum(W3 * r5)) - m0) <= tol * a0


def test_full_size_fp32_within_tolerance(solver_for):
    cfg = config2_with_pulse()
    out = []
    for prec in (64, 32):
        s = solver_for(dict(cfg, PRECISION=prec))
        s.step(cfg["DT"], 20)
        out.append(s.state()[0])
        s.close()
    p64, p32 = pressure(cfg, out[0]), pressure(cfg, out[1])
    assert np.linalg.norm(p32 - p64) <= 1e-5 * np.linalg.norm(p64)


def test_full_size_batch_matches_single_problems():
    """All 256 problems of config 4 (82.6 M nodes) advanced together; a sample
    of each order agrees with the single-problem FP32 path (the batch applies
    1/w after the line sums, so agreement is to rounding, not bitwise)."""
    W = workloads()
    m = dg()
    cfgs = W.config4(seed=0)
    steps = 20
    with m.Batch(cfgs) as b:
        b.step(steps)
        picks = {}
        for i, c in enumerate(cfgs):
            picks.setdefault(c["ORDER"], i)
        got = {i: b.state(i) for i in picks.values()}
    assert len(picks) == 4
    for i, (r, v) in got.items():
        c = cfgs[i]
        with m.Solver(c) as s:
            s.step(c["DT"], steps)
            r1, v1 = s.state()
        assert np.max(np.abs(r1)) > 0
        assert max_rel(pressure(c, r), pressure(c, r1)) <= 2e-5, (i, c["ORDER"])
        assert max_rel(v, v1) <= 2e-5
