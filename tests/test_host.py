"""Host-side (CPU-only) tests of libdg3d: the library loads and exports every
entry point of include/dg3d.h; the FP64 basis, the parameter parser and the
HDF5 writer.  No call here touches a GPU."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, dg, workloads

HEADER = os.path.join(ROOT, "include", "dg3d.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    m = dg()
    L = m.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", m.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (dg_\w+)", out))
    assert set(syms) <= exported, set(syms) - exported


def test_params_defaults_match_reference():
    m = dg()
    p = m.params_from_dict({})
    # driver.cpp:52-61 and BCParamDefault (cppsrc/BCParam.cpp:24)
    assert p.order == 4 and list(p.num_elements) == [4, 3, 2] and list(p.num_blocks) == [5, 4, 6]
    assert p.c0 == 1500.0 and p.rho0 == 1000.0 and p.b_over_a == 0.0
    assert list(p.sponge_width) == [10] * 6 and p.sigma_max == -1.0
    assert p.precision == 64 and p.src_face == -1


def test_parse_reference_format(tmp_path, capfd):
    m = dg()
    text = """#Total timesteps = Substeps * Outsteps
NUM_TIME_SUBSTEPS = 50
NUM_OUTSTEPS = 10
FREQ_TERMINAL = 10
ORDER = 3
ELEMENT_WIDTH = .125 .125 .25
STARTING_CORNER = -1.0 -1.0 -2.0
DT = 0.000001
C0 = 1500.0
DIFF_CONST = 5.0
RHO0 = 1000.0
B_OVER_A = 5.0
NUM_ELEMENTS = 8 8 16
NUM_BLOCKS = 2 2 1
EVALUATE_SPONGE = 1
EVALUATE_ADVECTION = 1
EVALUATE_DIFFUSION = 0
BC_IS_PERIODIC = 0 1 0
BC_SIGMA_MAX = 15000
BC_SPONGE_WIDTH = 1 2 3 4 5 6
IC_X_GAUSS = 1
IC_Y_GAUSS = 0
IC_Z_GAUSS = 1
IC_DRHO_AMPLITUDE = 1.0
IC_VX_AMPLITUDE = 0.5
IC_VY_AMPLITUDE = 0.0
IC_VZ_AMPLITUDE = 0.0
IC_SIGMA = 40.
IC_CENTER_X = 0.
IC_CENTER_Y = 0.25
IC_CENTER_Z = 0.
NOT_A_KEY = 3
"""
    pf = tmp_path / "p.txt"
    pf.write_text(text)
    log = tmp_path / "_log.txt"
    p, drv = m.parse_params(str(pf), str(log))
    assert drv == dict(DT=1e-6, NUM_TIME_SUBSTEPS=50, NUM_OUTSTEPS=10, FREQ_TERMINAL=10, BOOL_FILE=1)
    assert p.order == 3 and list(p.elem_width) == [0.125, 0.125, 0.25] and list(p.corner) == [-1.0, -1.0, -2.0]
    assert list(p.num_elements) == [8, 8, 16] and list(p.num_blocks) == [2, 2, 1]
    assert (p.eval_sponge, p.eval_advect, p.eval_diff) == (1, 1, 0)
    assert list(p.periodic) == [0, 1, 0] and p.sigma_max == 15000.0
    assert list(p.sponge_width) == [1, 2, 3, 4, 5, 6]
    assert list(p.ic_gauss) == [1, 0, 1] and p.ic_sigma == 40.0 and p.ic_v_amp[0] == 0.5
    assert p.ic_center[1] == 0.25 and p.diff_const == 5.0
    # log echo as the reference's driver writes it (cppsrc/driver.cpp:138-188)
    lg = log.read_text()
    assert lg.startswith("Parameters used:\n{\n  #Total timesteps") and lg.endswith("  NOT_A_KEY = 3\n}\n")
    err = capfd.readouterr().err
    assert 'WARNING: IGNORING INVALID PARAMETER LINE: "NOT_A_KEY = 3"' in err


def test_parse_missing_file_is_io_error():
    m = dg()
    with pytest.raises(m.DGError, match="Unable to open parameter file"):
        m.parse_params("/nonexistent/params.txt")


@pytest.mark.parametrize("order", range(1, 9))
def test_basis_matches_independent_generator(order):
    import refinputs
    m = dg()
    ops = m.line_operators(order)
    x, w = refinputs.lgl(order + 1)
    M, S = refinputs.unit_matrices(order)
    assert np.allclose(ops["zeros"], x, atol=2e-15, rtol=0)
    assert np.allclose(ops["mass"], M, atol=1e-15, rtol=1e-13)
    assert np.allclose(ops["stiff"], S, atol=1e-14, rtol=1e-13)
    K = order + 1
    # summation-by-parts: S + S^T = diag(-1, 0, ..., 0, 1)
    B = np.zeros((K, K))
    B[0, 0], B[-1, -1] = -1.0, 1.0
    assert np.allclose(ops["stiff"] + ops["stiff"].T, B, atol=1e-13)
    # D = M^-1 S and the lift columns
    assert np.allclose(ops["mass"] @ ops["deriv"], ops["stiff"], atol=1e-13)
    assert np.allclose(ops["mass"] @ ops["lift0"], np.eye(K)[0], atol=1e-12)
    assert np.allclose(ops["mass"] @ ops["liftN"], np.eye(K)[-1], atol=1e-12)


def test_lumped_mass_is_lgl_weights():
    m = dg()
    ops = m.line_operators(4, lumped=True)
    import refinputs
    _, w = refinputs.lgl(5)
    assert np.allclose(ops["mass"], np.diag(0.5 * w), atol=1e-16)


def test_basis_files_roundtrip(tmp_path):
    """Files written by the C ABI parse back (as the reference parses them)
    to the operators the C ABI computes."""
    m = dg()
    m.write_basis_files(str(tmp_path), kmax=10)
    import refinputs
    for order in (1, 3, 4, 7):
        M, S = refinputs.read_matrices(str(tmp_path / "matrices.txt"), order)
        z = refinputs.read_zeros(str(tmp_path / "hardcoded_coeff.txt"), order)
        ops = m.line_operators(order)
        assert np.array_equal(M, ops["mass"]) and np.array_equal(S, ops["stiff"])
        assert np.array_equal(z, ops["zeros"])
        ops2 = m.line_operators(order, matrix_file=str(tmp_path / "matrices.txt"),
                                coeff_file=str(tmp_path / "hardcoded_coeff.txt"))
        assert np.array_equal(ops2["mass"], M) and np.array_equal(ops2["zeros"], z)


def test_basis_reads_golden_files_exactly():
    import refinputs
    m = dg()
    g = os.path.join(ROOT, "tests", "golden")
    ops = m.line_operators(3, matrix_file=os.path.join(g, "matrices.txt"),
                           coeff_file=os.path.join(g, "hardcoded_coeff.txt"))
    M, S = refinputs.read_matrices(os.path.join(g, "matrices.txt"), 3)
    assert np.array_equal(ops["mass"], M) and np.array_equal(ops["stiff"], S)


def test_missing_matrix_file_is_io_error(tmp_path):
    m = dg()
    with pytest.raises(m.DGError, match="doesn't exist or is not accessible"):
        m.line_operators(3, matrix_file=str(tmp_path / "nope.txt"))


def test_order_out_of_range_rejected():
    m = dg()
    with pytest.raises(m.DGError):
        m.line_operators(0)


@pytest.mark.parametrize("order", [0, 8])
def test_solver_order_outside_kernels_rejected_at_create(order):
    """The kernels cover 2..8 nodes per line: other orders fail in dg_create,
    before any device work, not at the first step."""
    m = dg()
    cfg = workloads().gaussian_pulse(num_elements=(2, 2, 2), order=3)
    cfg["ORDER"] = order
    with pytest.raises(m.DGError, match="ORDER must be in 1..7"):
        m.Solver(cfg)


def test_hdf5_roundtrip(tmp_path):
    import importlib
    h5 = importlib.import_module("3ddg_gb300.h5read")
    m = dg()
    rng = np.random.default_rng(0)
    vec = rng.standard_normal((3, 5, 4, 6))
    sca = rng.standard_normal((7, 3, 2))
    m.hdf5_write(str(tmp_path / "vel_0_0.h5"), "velocity", vec, 1.25)
    m.hdf5_write(str(tmp_path / "dRho_0_0.h5"), "rho", sca, 2.5)
    d = h5.read(str(tmp_path / "vel_0_0.h5"))
    assert set(d) == {"velocity", "time"}
    assert np.array_equal(d["velocity"], vec) and d["time"].tolist() == [1.25]
    d = h5.read(str(tmp_path / "dRho_0_0.h5"))
    assert np.array_equal(d["rho"], sca) and d["time"].tolist() == [2.5]
    raw = open(tmp_path / "dRho_0_0.h5", "rb").read()
    assert raw[:8] == b"\x89HDF\r\n\x1a\n"


def test_hdf5_bad_path_is_reference_error_code(tmp_path):
    m = dg()
    with pytest.raises(m.DGError, match=r"\(-1\).*FileIException"):
        m.hdf5_write(str(tmp_path / "no" / "such" / "dir.h5"), "rho", np.zeros((2, 2, 2)))


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No fallback: with libdg3d.so absent, the first call raises DGError
    instead of running anything else."""
    m = dg()
    monkeypatch.setattr(m, "LIB_PATH", str(tmp_path / "libdg3d.so"))
    monkeypatch.setattr(m, "_lib", None)
    with pytest.raises(m.DGError, match="not built"):
        m.lib()
    with pytest.raises(m.DGError):
        m.Solver(workloads().config1(seed=0))
