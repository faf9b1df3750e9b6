"""Size-independent properties of the C oracle's right-hand side, beside its
pin to the reference's golden vectors (tests/test_oracle_golden.py): the
operator is affine in the state when the flux is linear (B/A = 0; diffusion
and sponge are linear), and the equations are symmetric under the mirror of
a mesh and sponges symmetric about the origin along each axis (with the
normal velocity changing sign), for the full nonlinear, diffusive, sponged
operator.  The mirror cases check the orientation of every face coefficient
and lift column along each axis (cppsrc/Element.cpp:542-600).  CPU only."""
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")


def base_cfg(order, ne, b_over_a):
    w = 1.25
    return {
        "BC_IS_PERIODIC": [0, 0, 0], "BC_SIGMA_MAX": 0.5, "BC_SPONGE_WIDTH": [1, 1, 1, 0, 0, 1],
        "B_OVER_A": b_over_a, "C0": 1.5, "DIFF_CONST": 4.3e-3, "DT": 0.02,
        "ELEMENT_WIDTH": [w, w, w], "EVALUATE_ADVECTION": 1, "EVALUATE_DIFFUSION": 1, "EVALUATE_SPONGE": 1,
        "IC_CENTER_X": 0.0, "IC_CENTER_Y": 0.0, "IC_CENTER_Z": 0.0, "IC_DRHO_AMPLITUDE": 0.0, "IC_SIGMA": 0.5,
        "IC_VX_AMPLITUDE": 0.0, "IC_VY_AMPLITUDE": 0.0, "IC_VZ_AMPLITUDE": 0.0,
        "IC_X_GAUSS": 1, "IC_Y_GAUSS": 1, "IC_Z_GAUSS": 1, "NUM_BLOCKS": [1, 1, 1], "NUM_ELEMENTS": list(ne),
        "ORDER": order, "RHO0": 1000.0, "STARTING_CORNER": [-0.5 * ne[0] * w, -0.5 * ne[1] * w, -0.5 * ne[2] * w],
    }


def oracle(cfg):
    import pyoracle
    import refinputs
    order = int(cfg["ORDER"])
    M, S = refinputs.read_matrices(os.path.join(GOLDEN, "matrices.txt"), order)
    z = refinputs.read_zeros(os.path.join(GOLDEN, "hardcoded_coeff.txt"), order)
    return pyoracle.Oracle(cfg, M, S, z)


def rhs_of(o, rho, vel):
    o.set_state(rho, vel)
    return o.rhs()


def random_state(o, rng, scale=1e-3):
    shape = o.state()[0].shape
    return rng.standard_normal(shape) * scale, rng.standard_normal((3,) + shape) * scale * 1e-3


@pytest.mark.parametrize("order", [1, 2, 4])
def test_rhs_is_affine_with_linear_flux(order):
    o = oracle(base_cfg(order, (3, 2, 3), 0.0))
    rng = np.random.default_rng(order)
    u, v = random_state(o, rng), random_state(o, rng)
    a, b = 0.7, -1.9
    r0 = rhs_of(o, np.zeros_like(u[0]), np.zeros_like(u[1]))
    ru, rv = rhs_of(o, *u), rhs_of(o, *v)
    rw = rhs_of(o, a * u[0] + b * v[0], a * u[1] + b * v[1])
    for f in range(2):
        want = a * (ru[f] - r0[f]) + b * (rv[f] - r0[f])
        got = rw[f] - r0[f]
        assert np.max(np.abs(got - want)) <= 1e-10 * np.max(np.abs(want))
    o.close()


def mirror(rho, vel, axis):
    """Reflection of the node grid along ``axis`` (LGL nodes are symmetric,
    so node i of the grid maps to node X - 1 - i), the normal velocity
    component changing sign."""
    rho_m = np.flip(rho, axis).copy()
    vel_m = np.flip(vel, axis + 1).copy()
    vel_m[axis] *= -1.0
    return rho_m, vel_m


@pytest.mark.parametrize("order,axis", [(2, 0), (3, 0), (3, 1), (2, 2), (4, 1)])
def test_rhs_is_mirror_symmetric(order, axis):
    """Sponges of one element on all six faces, a mesh centred on the origin:
    the operator commutes with the reflection of the node grid along each
    axis."""
    cfg = base_cfg(order, (4, 2, 3), 5.0)
    cfg["BC_SPONGE_WIDTH"] = [1] * 6
    o = oracle(cfg)
    rng = np.random.default_rng(10 + order + 3 * axis)
    rho, vel = random_state(o, rng)
    r, v = rhs_of(o, rho, vel)
    rm, vm = rhs_of(o, *mirror(rho, vel, axis))
    want_r, want_v = mirror(r, v, axis)
    assert np.max(np.abs(rm - want_r)) <= 1e-12 * np.max(np.abs(r))
    assert np.max(np.abs(vm - want_v)) <= 1e-12 * np.max(np.abs(v))
    # the check has teeth: the unmirrored state gives a different field
    assert np.max(np.abs(rm - r)) > 1e-3 * np.max(np.abs(r))
    o.close()
