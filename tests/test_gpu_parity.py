"""GPU FP64 path against the C oracle on identical seeded inputs, through the
C ABI.  Tolerances: one right-hand-side evaluation to 1e-12 relative (rounding
only), multi-step runs to 1e-10 max relative pressure error."""
import numpy as np
import pytest

from conftest import dg, max_rel, pressure, workloads

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
STEP_TOL = 1e-10


def small(order=3, ne=(4, 3, 5), **kw):
    W = workloads()
    cfg = W.gaussian_pulse(seed=1, num_elements=ne, order=order, width=1.25, sponge=1, **kw)
    cfg["IC_CENTER_X"] = 0.3  # off-centre so every axis sees asymmetric data
    cfg["IC_CENTER_Y"] = -0.2
    cfg["IC_CENTER_Z"] = 0.1
    cfg["IC_VX_AMPLITUDE"] = 0.001
    cfg["IC_VZ_AMPLITUDE"] = -0.0005
    cfg["DT"] = W.cfl_dt(cfg)
    return cfg


def compare_state(cfg, s, o, tol):
    r_g, v_g = s.state()
    r_o, v_o = o.state()
    ep = max_rel(pressure(cfg, r_g), pressure(cfg, r_o))
    ev = max_rel(v_g, v_o)
    assert ep <= tol and ev <= tol, (ep, ev)
    return ep, ev


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6, 7])
def test_rhs_matches_oracle(order, solver_for, oracle_for):
    cfg = small(order=order)
    s, o = solver_for(cfg), oracle_for(cfg)
    r_g, v_g = s.rhs()
    r_o, v_o = o.rhs()
    assert max_rel(r_g, r_o) <= RHS_TOL
    for a in range(3):
        assert max_rel(v_g[a], v_o[a]) <= RHS_TOL


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_steps_match_oracle(order, solver_for, oracle_for):
    cfg = small(order=order)
    s, o = solver_for(cfg), oracle_for(cfg)
    s.step(cfg["DT"], 6)
    o.run(cfg["DT"], 6)
    compare_state(cfg, s, o, STEP_TOL)
    assert abs(s.time - o.time) < 1e-15


def test_config1_short_matches_oracle(solver_for, oracle_for):
    cfg = workloads().config1(seed=0)
    s, o = solver_for(cfg), oracle_for(cfg)
    s.step(cfg["DT"], 10)
    o.run(cfg["DT"], 10)
    compare_state(cfg, s, o, STEP_TOL)


# N = 4 runs the FP64 kernels with even-odd line owners, N = 3 with per-node line sums.
@pytest.mark.parametrize("order,periodic", [(3, (1, 0, 0)), (3, (0, 1, 1)), (3, (1, 1, 1)), (4, (1, 0, 1)),
                                            (4, (1, 1, 1))])
def test_periodic_matches_oracle(order, periodic, solver_for, oracle_for):
    cfg = small(order=order, periodic=periodic)
    s, o = solver_for(cfg), oracle_for(cfg)
    s.step(cfg["DT"], 5)
    o.run(cfg["DT"], 5)
    compare_state(cfg, s, o, STEP_TOL)


@pytest.mark.parametrize("order", [3, 4])
def test_no_diffusion_no_sponge(order, solver_for, oracle_for):
    cfg = small(order=order, diffusion=False)
    cfg["EVALUATE_SPONGE"] = 0
    s, o = solver_for(cfg), oracle_for(cfg)
    s.step(cfg["DT"], 5)
    o.run(cfg["DT"], 5)
    compare_state(cfg, s, o, STEP_TOL)


@pytest.mark.parametrize("order", [3, 4])
def test_diffusion_only(order, solver_for, oracle_for):
    """EVALUATE_ADVECTION = 0: no volume fluxes (no flux buffers), the line
    owners skip the momentum lines; FP32 against FP64 as well."""
    cfg = small(order=order)
    cfg["EVALUATE_ADVECTION"] = 0
    cfg["DIFF_CONST"] = 0.05
    s, o = solver_for(cfg), oracle_for(cfg)
    s.step(cfg["DT"], 5)
    o.run(cfg["DT"], 5)
    compare_state(cfg, s, o, STEP_TOL)
    r0, _ = o.state()
    assert np.max(np.abs(r0)) > 0
    s32 = solver_for(dict(cfg, PRECISION=32))
    s32.step(cfg["DT"], 5)
    r64, _ = s.state()
    r32, _ = s32.state()
    assert np.linalg.norm(r32 - r64) <= 1e-5 * np.linalg.norm(r64)


@pytest.mark.parametrize("order", [3, 4])
def test_linear_mass_flux(order, solver_for, oracle_for):
    cfg = small(order=order)
    cfg["B_OVER_A"] = 0.0
    s, o = solver_for(cfg), oracle_for(cfg)
    s.step(cfg["DT"], 5)
    o.run(cfg["DT"], 5)
    compare_state(cfg, s, o, STEP_TOL)


@pytest.mark.parametrize("order", [3, 4])
def test_multiblock_equivalent_to_single_block(order, solver_for, oracle_for):
    """2x2x2 blocks with the on-device face gather == one block of the same
    global mesh (the reference's MPI exchange makes them identical)."""
    cfg1 = small(order=order, ne=(6, 4, 6))
    cfg8 = dict(cfg1)
    cfg8["NUM_ELEMENTS"] = [3, 2, 3]
    cfg8["NUM_BLOCKS"] = [2, 2, 2]
    s1, s8 = solver_for(cfg1), solver_for(cfg8)
    rng = np.random.default_rng(3)
    r = rng.standard_normal(s1.dims) * 1e-3
    v = rng.standard_normal((3,) + s1.dims) * 1e-6
    s1.set_state(r, v)
    s8.set_state(r, v)
    s1.step(cfg1["DT"], 4)
    s8.step(cfg1["DT"], 4)
    r1, v1 = s1.state()
    r8, v8 = s8.state()
    assert np.array_equal(r1, r8) and np.array_equal(v1, v8)
    # and the multi-block IC run matches the oracle
    o = oracle_for(cfg8)
    s = solver_for(cfg8)
    s.step(cfg8["DT"], 4)
    o.run(cfg8["DT"], 4)
    compare_state(cfg8, s, o, STEP_TOL)


@pytest.mark.parametrize("order", [3, 4])
def test_tone_burst_source_matches_oracle(order, solver_for, oracle_for):
    W = workloads()
    cfg = W.scaled(W.config2(seed=0), (6, 6, 8))
    cfg["ORDER"] = order
    cfg["SRC_RADIUS"] = 1.2
    cfg["DT"] = W.cfl_dt(cfg)
    s, o = solver_for(cfg), oracle_for(cfg)
    n = 40
    s.step(cfg["DT"], n)
    o.run(cfg["DT"], n)
    r, _ = o.state()
    assert np.max(np.abs(r)) > 1e-3  # the burst has entered the domain
    compare_state(cfg, s, o, STEP_TOL)


def test_set_state_clears_ic_halo(solver_for, oracle_for):
    cfg = small(order=2)
    s, o = solver_for(cfg), oracle_for(cfg)
    r, v = o.state()
    s.set_state(r, v)
    o.set_state(r, v)
    s.step(cfg["DT"], 3)
    o.run(cfg["DT"], 3)
    compare_state(cfg, s, o, STEP_TOL)


@pytest.mark.parametrize("order", [3, 4])
def test_anisotropic_elements_match_oracle(order, solver_for, oracle_for):
    """Different element widths per axis: the per-axis operator scales (and,
    at N = 4, the line owners' per-axis coefficients picked by a runtime axis)
    must not mix axes."""
    W = workloads()
    cfg = small(order=order, ne=(4, 5, 3))
    cfg["ELEMENT_WIDTH"] = [1.25, 0.9, 1.6]
    cfg["STARTING_CORNER"] = [-2.5, -2.25, -2.4]
    cfg["IC_VY_AMPLITUDE"] = 0.0007
    cfg["DT"] = W.cfl_dt(cfg)
    s, o = solver_for(cfg), oracle_for(cfg)
    s.step(cfg["DT"], 5)
    o.run(cfg["DT"], 5)
    compare_state(cfg, s, o, STEP_TOL)
    s32 = solver_for(dict(cfg, PRECISION=32))
    s32.step(cfg["DT"], 5)
    r64, _ = s.state()
    r32, _ = s32.state()
    assert np.linalg.norm(r32 - r64) <= 1e-5 * np.linalg.norm(r64)


@pytest.mark.parametrize("order", [3, 4])
def test_lumped_mass_matches_oracle(order, tmp_path):
    """Diagonal (LGL-lumped) mass matrices: a different D and lift columns
    that are zero away from the line ends; both sides read the same files."""
    import pyoracle
    import refinputs
    refinputs.write_coeff_files(str(tmp_path))
    refinputs.write_matrices(str(tmp_path), lumped=True)
    mf, cf = str(tmp_path / "matrices.txt"), str(tmp_path / "hardcoded_coeff.txt")
    cfg = small(order=order)
    M, S = refinputs.read_matrices(mf, order)
    assert np.count_nonzero(M - np.diag(np.diag(M))) == 0
    o = pyoracle.Oracle(cfg, M, S, refinputs.read_zeros(cf, order))
    with dg().Solver(cfg, mf, cf) as s:
        s.step(cfg["DT"], 5)
        o.run(cfg["DT"], 5)
        compare_state(cfg, s, o, STEP_TOL)


def test_operator_without_mirror_symmetry_matches_oracle(tmp_path):
    """The N = 4 kernels' even-odd line owners need D to be centro-
    antisymmetric; a matrix file whose S breaks that (one entry scaled by
    1 + 1e-6) must take the per-node line sums and still match the oracle
    running the same operator."""
    import pyoracle
    import refinputs
    refinputs.write_coeff_files(str(tmp_path))
    with open(tmp_path / "matrices.txt", "w") as f:
        for N in range(1, refinputs.KMAX):
            M, S = refinputs.unit_matrices(N, False)
            S = np.array(S, dtype=np.float64)
            if N == 4:
                S[0, 1] *= 1.0 + 1e-6
            f.write("Order=%d\n" % N)
            for r in np.asarray(M):
                f.write(" ".join(refinputs.hexd(v) for v in r) + "\n")
            for r in S:
                f.write(" ".join(refinputs.hexd(v) for v in r) + "\n")
    mf, cf = str(tmp_path / "matrices.txt"), str(tmp_path / "hardcoded_coeff.txt")
    cfg = small(order=4)
    M, S = refinputs.read_matrices(mf, 4)
    assert abs(S[0][1] + S[4][3]) > 1e-8 * abs(S[0][1])  # the mirror symmetry is broken
    o = pyoracle.Oracle(cfg, M, S, refinputs.read_zeros(cf, 4))
    with dg().Solver(cfg, mf, cf) as s:
        s.step(cfg["DT"], 5)
        o.run(cfg["DT"], 5)
        compare_state(cfg, s, o, STEP_TOL)


@pytest.mark.parametrize("order,kw", [(2, {}), (4, {"periodic": (1, 0, 1)}), (3, {"diffusion": False})])
def test_flux_buffers_bitwise_after_state_round_trip(order, kw, solver_for):
    """FP64 stages read their input's volume fluxes (and the neighbours') from
    the buffer the previous stage wrote; after set_state the first stage
    evaluates them from the state instead.  Both evaluate the same FP64
    expressions of the same values, so a state round trip between steps
    changes no bit."""
    cfg = small(order=order, **kw)
    a, b = solver_for(cfg), solver_for(cfg)
    a.step(cfg["DT"], 1)
    b.step(cfg["DT"], 1)
    a.step(cfg["DT"], 3)
    for _ in range(3):
        r, v = b.state()
        b.set_state(r, v)
        b.step(cfg["DT"], 1)
    ra, va = a.state()
    rb, vb = b.state()
    assert np.max(np.abs(ra)) > 0 and np.max(np.abs(va)) > 0
    assert np.array_equal(ra, rb) and np.array_equal(va, vb)


def test_state_written_in_device_memory_is_seen_by_the_next_step(solver_for):
    """dg_state_device hands out the state for zero-copy coupling: a state
    written through it (here halved in place by torch) must be stepped from
    its own volume fluxes, not the ones cached for the old state, exactly as
    the same state set through dg_set_state."""
    import torch

    class DeviceArray:
        def __init__(self, ptr, n):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 2}

    cfg = small(order=4)
    a, b = solver_for(cfg), solver_for(cfg)
    a.step(cfg["DT"], 2)
    b.step(cfg["DT"], 2)
    base, NP, n_elem = a.device_state()
    a.synchronize()
    for f in range(4):
        torch.as_tensor(DeviceArray(base[f], n_elem * NP), device="cuda").mul_(0.5)
    torch.cuda.synchronize()
    r, v = b.state()
    b.set_state(0.5 * r, 0.5 * v)
    a.step(cfg["DT"], 2)
    b.step(cfg["DT"], 2)
    ra, va = a.state()
    rb, vb = b.state()
    assert np.max(np.abs(ra)) > 0
    assert np.array_equal(ra, rb) and np.array_equal(va, vb)


@pytest.mark.parametrize("precision", [64, 32])
def test_pinned_host_buffers_match_pageable(precision, solver_for):
    """Pinned host buffers are read/written by the kernels directly; pageable
    ones go through device staging.  Both give the same bytes."""
    import torch
    cfg = small(order=3, ne=(3, 4, 2))
    cfg["PRECISION"] = precision
    s = solver_for(cfg)
    s.step(cfg["DT"], 3)
    r, v = s.state()
    rp = torch.empty(r.shape, dtype=torch.float64, pin_memory=True).numpy()
    vp = torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy()
    s.state(rp, vp)
    assert np.array_equal(r, rp) and np.array_equal(v, vp)
    rp[...] = r * 1.5
    vp[...] = v * 0.5
    s.set_state(rp, vp)
    r2, v2 = s.state()
    tol = 0 if precision == 64 else 1e-6
    assert np.allclose(r2, rp, rtol=tol, atol=0) and np.allclose(v2, vp, rtol=tol, atol=0)


@pytest.mark.parametrize("precision", [64, 32])
def test_probe_records_pressure_at_nearest_node(precision, solver_for):
    cfg = small(order=3)
    cfg["PRECISION"] = precision
    s = solver_for(cfg)
    pts = np.array([[0.3, -0.2, 0.1], [100.0, 100.0, -100.0]])
    s.probe_set(pts)
    for _ in range(3):
        s.step(cfg["DT"], 2)
    t, p = s.probe_get()
    assert p.shape == (6, 2) and np.all(np.diff(t) > 0) and abs(t[-1] - s.time) < 1e-15
    r, _ = s.state()
    c, _ = s.grid()
    for k, x in enumerate(pts):
        d2 = sum((c[a] - x[a]) ** 2 for a in range(3))
        idx = np.unravel_index(np.argmin(d2), d2.shape)
        assert abs(p[-1, k] - pressure(cfg, r[idx])) <= 1e-12 * max(1.0, abs(p[-1, k]))


def test_fp32_form_within_tolerance(solver_for, oracle_for):
    """FP32 fields/fluxes/stages with the Kahan-compensated update against the
    FP64 oracle: relative L2 pressure error <= 1e-5."""
    cfg = workloads().config1(seed=0)
    cfg32 = dict(cfg)
    cfg32["PRECISION"] = 32
    s, o = solver_for(cfg32), oracle_for(cfg)
    n = 50
    s.step(cfg["DT"], n)
    o.run(cfg["DT"], n)
    r_g, _ = s.state()
    r_o, _ = o.state()
    p_g, p_o = pressure(cfg, r_g), pressure(cfg, r_o)
    l2 = np.linalg.norm(p_g - p_o) / np.linalg.norm(p_o)
    assert l2 <= 1e-5, l2


@pytest.mark.parametrize("precision", [64, 32])
def test_async_transfers_match_sync(precision, solver_for):
    """dg_set_state_async / dg_get_state_async pipelined over several steps give
    the same bytes as the synchronous calls; pageable buffers are refused."""
    import torch
    m = __import__("conftest").dg()
    cfg = small(order=3, ne=(3, 4, 2))
    cfg["PRECISION"] = precision
    a, b = solver_for(cfg), solver_for(cfg)
    shape = a.dims
    rng = np.random.default_rng(11)

    def pinned(shp):
        return torch.empty(shp, dtype=torch.float64, pin_memory=True).numpy()

    ins, outs = [], []
    for k in range(3):
        r, v = pinned(shape), pinned((3,) + shape)
        r[...] = rng.standard_normal(shape) * 1e-3
        v[...] = rng.standard_normal((3,) + shape) * 1e-6
        ins.append((r, v))
        outs.append((pinned(shape), pinned((3,) + shape)))
    for k in range(3):
        a.set_state_async(*ins[k])
        a.step(cfg["DT"], 2)
        a.state_async(*outs[k])
    a.synchronize()
    for k in range(3):
        b.set_state(*ins[k])
        b.step(cfg["DT"], 2)
        r, v = b.state()
        assert np.array_equal(r, outs[k][0]) and np.array_equal(v, outs[k][1])
    with pytest.raises(m.DGError, match="page-locked"):
        a.set_state_async(np.zeros(shape), np.zeros((3,) + shape))
    with pytest.raises(m.DGError, match="page-locked"):
        a.state_async(np.zeros(shape), None)


@pytest.mark.parametrize("precision", [64, 32])
def test_async_transfers_ordering(precision, solver_for):
    """Downloads between steps without uploads (the step waits for the pack of
    the buffer it writes), a download right after an upload, and synchronous
    calls mixed in: every download holds the state at its place in the call
    sequence."""
    import torch
    cfg = small(order=2, ne=(3, 3, 4))
    cfg["PRECISION"] = precision
    a, b = solver_for(cfg), solver_for(cfg)
    shape = a.dims
    rng = np.random.default_rng(5)

    def pinned(shp):
        return torch.empty(shp, dtype=torch.float64, pin_memory=True).numpy()

    r0, v0 = pinned(shape), pinned((3,) + shape)
    r0[...] = rng.standard_normal(shape) * 1e-3
    v0[...] = rng.standard_normal((3,) + shape) * 1e-6
    outs = [(pinned(shape), pinned((3,) + shape)) for _ in range(5)]
    a.set_state_async(r0, v0)
    a.state_async(*outs[0])           # right after the upload
    for k in range(1, 4):
        a.step(cfg["DT"], 1)
        a.state_async(*outs[k])       # no upload in between
    r_sync, v_sync = a.state()        # synchronous read in the mix
    a.set_state(r_sync, v_sync)       # synchronous write after an async download
    a.step(cfg["DT"], 1)
    a.state_async(*outs[4])
    a.synchronize()
    b.set_state(r0, v0)
    exp = [b.state()]
    for k in range(1, 4):
        b.step(cfg["DT"], 1)
        exp.append(b.state())
    b.set_state(*exp[3])  # as a does (in FP32 this also clears the Kahan compensation)
    b.step(cfg["DT"], 1)
    exp.append(b.state())
    for k in range(5):
        assert np.array_equal(outs[k][0], exp[k][0]) and np.array_equal(outs[k][1], exp[k][1]), k
    assert np.array_equal(r_sync, exp[3][0])


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6, 7])
def test_fp32_every_order_within_tolerance(order, solver_for):
    """FP32 form (per-node line sums for K <= 4, line owners above) against the
    FP64 path on the same inputs: relative L2 pressure error <= 1e-5."""
    cfg = small(order=order, ne=(4, 3, 4))
    s64 = solver_for(cfg)
    s32 = solver_for(dict(cfg, PRECISION=32))
    for s in (s64, s32):
        s.step(cfg["DT"], 10)
    r64, v64 = s64.state()
    r32, v32 = s32.state()
    p64, p32 = pressure(cfg, r64), pressure(cfg, r32)
    assert np.linalg.norm(p32 - p64) <= 1e-5 * np.linalg.norm(p64)
    assert np.linalg.norm(v32 - v64) <= 1e-5 * np.linalg.norm(v64)


@pytest.mark.parametrize("ne,periodic,order", [((1, 1, 1), (0, 0, 0), 3), ((1, 2, 3), (1, 1, 1), 4),
                                               ((2, 1, 1), (1, 0, 0), 4), ((1, 1, 2), (0, 0, 1), 5),
                                               ((1, 1, 1), (0, 0, 0), 4), ((3, 1, 1), (1, 0, 0), 4)])
def test_tiny_meshes_match_oracle(ne, periodic, order, solver_for, oracle_for):
    """One element along an axis: with a periodic axis the element is its own
    neighbour across that axis (the reference's periodicSelf copies its own
    opposite face).  FP64 against the oracle; FP32 against FP64.  Odd element
    counts at N = 4 leave the last CTA of the two-element line-owner kernels
    half empty."""
    cfg = small(order=order, ne=ne, periodic=periodic)
    cfg["EVALUATE_SPONGE"] = 0
    s, o = solver_for(cfg), oracle_for(cfg)
    s.step(cfg["DT"], 4)
    o.run(cfg["DT"], 4)
    compare_state(cfg, s, o, STEP_TOL)
    s32 = solver_for(dict(cfg, PRECISION=32))
    s32.step(cfg["DT"], 4)
    r64, _ = s.state()
    r32, _ = s32.state()
    p64, p32 = pressure(cfg, r64), pressure(cfg, r32)
    assert np.linalg.norm(p32 - p64) <= 1e-5 * np.linalg.norm(p64)


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("order,ne,nb", [(1, (2, 3, 19), (1, 1, 1)), (2, (3, 2, 17), (2, 1, 2)),
                                         (3, (2, 2, 9), (1, 2, 2)), (4, (3, 2, 18), (2, 2, 1)),
                                         (5, (2, 3, 9), (1, 1, 2)), (6, (2, 2, 5), (2, 1, 1)),
                                         (7, (2, 1, 5), (1, 1, 2))])
def test_set_state_round_trip_every_order(order, ne, nb, precision, solver_for):
    """dg_set_state from pageable memory goes through device staging and the
    element-order unpack into the element-major state (multi-block meshes,
    z extents that are not multiples of a tile); reading it back gives the
    same values (FP64: bitwise; FP32: the values rounded to float)."""
    cfg = small(order=order, ne=ne)
    cfg["NUM_BLOCKS"] = list(nb)
    cfg["PRECISION"] = precision
    s = solver_for(cfg)
    X, Y, Z = s.dims
    rng = np.random.default_rng(order)
    r = rng.standard_normal((X, Y, Z))
    v = rng.standard_normal((3, X, Y, Z))
    s.set_state(r, v)
    r2, v2 = s.state()
    if precision == 64:
        assert np.array_equal(r2, r) and np.array_equal(v2, v)
    else:
        assert np.array_equal(r2, r.astype(np.float32).astype(np.float64))
        assert np.array_equal(v2, v.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("precision,advect", [(64, 1), (64, 0), (32, 1)])
def test_async_uploads_back_to_back(precision, advect, solver_for):
    """Asynchronous uploads land in a spare state buffer that is swapped in at
    their place in the call sequence: two uploads in a row (the second reuses
    the buffer the first swapped out), a step, a download, then an upload
    followed at once by a download, give what the synchronous calls give.
    With advection off there are no volume-flux buffers to swap."""
    import torch
    cfg = small(order=3, ne=(2, 3, 3))
    cfg["PRECISION"] = precision
    cfg["EVALUATE_ADVECTION"] = advect
    a, b = solver_for(cfg), solver_for(cfg)
    shape = a.dims
    rng = np.random.default_rng(3)

    def pinned(shp):
        return torch.empty(shp, dtype=torch.float64, pin_memory=True).numpy()

    A = (pinned(shape), pinned((3,) + shape))
    B = (pinned(shape), pinned((3,) + shape))
    for r, v in (A, B):
        r[...] = rng.standard_normal(shape) * 1e-3
        v[...] = rng.standard_normal((3,) + shape) * 1e-6
    out1 = (pinned(shape), pinned((3,) + shape))
    out2 = (pinned(shape), pinned((3,) + shape))
    a.set_state_async(*A)
    a.set_state_async(*B)
    a.step(cfg["DT"], 2)
    a.state_async(*out1)
    a.set_state_async(*A)
    a.state_async(*out2)
    a.step(cfg["DT"], 1)
    a.synchronize()
    b.set_state(*B)
    b.step(cfg["DT"], 2)
    r1, v1 = b.state()
    assert np.array_equal(out1[0], r1) and np.array_equal(out1[1], v1)
    b.set_state(*A)
    r2, v2 = b.state()
    assert np.array_equal(out2[0], r2) and np.array_equal(out2[1], v2)
    b.step(cfg["DT"], 1)
    ra, va = a.state()
    rb, vb = b.state()
    assert np.array_equal(ra, rb) and np.array_equal(va, vb)


@pytest.mark.parametrize("order,precision,advect,nb", [(3, 64, 1, (1, 1, 1)), (4, 64, 1, (2, 1, 2)),
                                                        (4, 64, 0, (1, 1, 1)), (3, 32, 1, (1, 1, 1))])
def test_step_and_download_matches_separate_calls(order, precision, advect, nb, solver_for):
    """dg_step_get_state_async (in the FP64 path with advection the last stage
    writes the host-order download itself) gives the bytes of dg_step followed
    by a download, through uploads, and leaves the state the same."""
    import torch
    cfg = small(order=order, ne=(2, 3, 4))
    cfg["NUM_BLOCKS"] = list(nb)
    cfg["PRECISION"] = precision
    cfg["EVALUATE_ADVECTION"] = advect
    a, b = solver_for(cfg), solver_for(cfg)
    shape = a.dims
    rng = np.random.default_rng(order + 7)

    def pinned(shp):
        return torch.empty(shp, dtype=torch.float64, pin_memory=True).numpy()

    ins = []
    for _ in range(3):
        r, v = pinned(shape), pinned((3,) + shape)
        r[...] = rng.standard_normal(shape) * 1e-3
        v[...] = rng.standard_normal((3,) + shape) * 1e-6
        ins.append((r, v))
    outs = [(pinned(shape), pinned((3,) + shape)) for _ in range(3)]
    for k in range(3):
        a.set_state_async(*ins[k])
        a.step(cfg["DT"], 1)
        a.step_state_async(cfg["DT"], *outs[k])
    a.synchronize()
    for k in range(3):
        b.set_state(*ins[k])
        b.step(cfg["DT"], 2)
        r, v = b.state()
        assert np.max(np.abs(r)) > 0
        assert np.array_equal(r, outs[k][0]) and np.array_equal(v, outs[k][1]), k
    ra, va = a.state()
    rb, vb = b.state()
    assert np.array_equal(ra, rb) and np.array_equal(va, vb)


@pytest.mark.parametrize("order,axis", [(2, 0), (3, 0), (4, 0), (4, 1), (4, 2), (3, 2)])
def test_rhs_is_mirror_symmetric(order, axis, solver_for):
    """The GPU right-hand side (nonlinear flux, LDG diffusion, sponge on all
    faces, mesh centred on the origin) commutes with the reflection of the
    node grid along each axis, the normal velocity changing sign: a check of
    every face coefficient's and lift column's orientation that does not go
    through the oracle (orders 2 and 4 use the even-odd line owners, 3 the
    per-node sums in the stage kernel)."""
    cfg = small(order=order, ne=(4, 3, 2))
    s = solver_for(cfg)
    X, Y, Z = s.dims
    rng = np.random.default_rng(20 + order + 3 * axis)
    rho = rng.standard_normal((X, Y, Z)) * 1e-3
    vel = rng.standard_normal((3, X, Y, Z)) * 1e-6

    def mirror(a, b):
        am, bm = np.flip(a, axis).copy(), np.flip(b, axis + 1).copy()
        bm[axis] *= -1.0
        return am, bm

    s.set_state(rho, vel)
    r, v = s.rhs()
    s.set_state(*mirror(rho, vel))
    rm, vm = s.rhs()
    want_r, want_v = mirror(r, v)
    assert np.max(np.abs(rm - want_r)) <= 1e-12 * np.max(np.abs(r))
    assert np.max(np.abs(vm - want_v)) <= 1e-12 * np.max(np.abs(v))
    assert np.max(np.abs(rm - r)) > 1e-3 * np.max(np.abs(r))
