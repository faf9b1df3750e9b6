import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdg3d.so")


def dg():
    return importlib.import_module("3ddg_gb300")


def workloads():
    return importlib.import_module("3ddg_gb300.workloads")


def pressure(cfg, drho):
    """p = c0^2 (drho + B/A / (2 rho0) drho^2): the equation of state of the
    momentum flux (cppsrc/kernelFuncs.cpp:15)."""
    c0, r0, ba = cfg["C0"], cfg["RHO0"], cfg["B_OVER_A"]
    return c0 * c0 * (drho + ba / (2.0 * r0) * drho * drho)


def max_rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


@pytest.fixture(scope="session")
def basis_dir(tmp_path_factory):
    """hardcoded_coeff.txt / matrices.txt written by the oracle-side generator
    (oracle/refinputs.py), shared by the GPU path and the oracle so both use
    bit-identical operators."""
    import refinputs
    d = tmp_path_factory.mktemp("basis")
    refinputs.write_coeff_files(str(d))
    refinputs.write_matrices(str(d))
    return str(d)


@pytest.fixture(scope="session")
def oracle_for(basis_dir):
    import pyoracle
    import refinputs

    def make(cfg):
        order = int(cfg["ORDER"])
        M, S = refinputs.read_matrices(os.path.join(basis_dir, "matrices.txt"), order)
        z = refinputs.read_zeros(os.path.join(basis_dir, "hardcoded_coeff.txt"), order)
        return pyoracle.Oracle(cfg, M, S, z)

    return make


@pytest.fixture(scope="session")
def solver_for(basis_dir):
    def make(cfg):
        m = dg()
        return m.Solver(cfg, os.path.join(basis_dir, "matrices.txt"), os.path.join(basis_dir, "hardcoded_coeff.txt"))

    return make
