"""dg_eval_rhs_noalloc: the right-hand-side evaluation for callers that
cannot allocate device memory (hosts that own all device memory through their
own pool or arena and therefore cannot create a dg_handle).  It keeps its LDG
gradient scratch in a static device array instead of an allocation.

Checked through the C ABI against the handle-based dg_eval_rhs on the same
state, twice in a row (the second call reuses the scratch left by the first),
within the one-evaluation tolerance of the other right-hand-side tests: orders
1..7, with and without diffusion, without sponge (no sigma buffer), and at
exactly the size limits.  This
file is collected last so that a run stopping at the first failure has already
run every other test."""
import ctypes as C

import numpy as np
import pytest

from conftest import dg, max_rel, workloads

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12


def face_table(ne):
    """Single-block face table in the library's element order, faces -X +X -Y
    +Y -Z +Z; boundary faces get slot = 6 e + f."""
    Ex, Ey, Ez = ne
    nbr = np.empty((Ex * Ey * Ez, 6), dtype=np.int32)
    for i in range(Ex):
        for j in range(Ey):
            for k in range(Ez):
                e = (i * Ey + j) * Ez + k
                for f in range(6):
                    a, side = f // 2, f % 2
                    g = [i, j, k]
                    g[a] += 1 if side else -1
                    if 0 <= g[a] < ne[a]:
                        nbr[e, f] = (g[0] * Ey + g[1]) * Ez + g[2]
                    else:
                        nbr[e, f] = -1 - (6 * e + f)
    return nbr


def to_grid(flat, ne, K, NP):
    """element-major [4][n_elem][NP] -> node-duplicated [4][X][Y][Z]."""
    Ex, Ey, Ez = ne
    a = flat.reshape(4, Ex, Ey, Ez, NP)[..., :K ** 3].reshape(4, Ex, Ey, Ez, K, K, K)
    return a.transpose(0, 1, 4, 2, 5, 3, 6).reshape(4, Ex * K, Ey * K, Ez * K)


def check_against_handle(cfg, ne, calls=2):
    """Evaluate the right-hand side of ``cfg``'s initial state with
    dg_eval_rhs_noalloc ``calls`` times in a row and compare every result with
    the handle-based dg_eval_rhs; the calls must agree bitwise."""
    import torch
    m = dg()
    K = int(cfg["ORDER"]) + 1
    with m.Solver(cfg) as s:
        r0, v0 = s.state()
        s.set_state(r0, v0)  # boundary exterior zero in both paths
        ref_rho, ref_vel = s.rhs()
        base, NP, n_elem = s.device_state()
        ops = m.line_operators(int(cfg["ORDER"]))
        d_nbr = torch.from_numpy(face_table(ne)).cuda()
        sponge = bool(s.params.eval_sponge)
        d_sig = None
        if sponge:
            _, sig_nodes = s.grid()
            sigma = sig_nodes[::K, ::K, ::K].reshape(-1).copy()  # one value per element, element order
            d_sig = torch.from_numpy(sigma).cuda()
        mass = np.ascontiguousarray(ops["mass"])
        stiff = np.ascontiguousarray(ops["stiff"])
        s.synchronize()
        outs = []
        for _ in range(calls):
            d_rhs = torch.full((4 * n_elem * NP,), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            rc = m.lib().dg_eval_rhs_noalloc(C.byref(s.params), mass.ctypes.data, stiff.ctypes.data, base[0],
                                             d_nbr.data_ptr(), d_sig.data_ptr() if sponge else None,
                                             d_rhs.data_ptr(), n_elem, None)
            assert rc == 0, m.lib().dg_last_error().decode()
            torch.cuda.synchronize()
            outs.append(to_grid(d_rhs.cpu().numpy(), ne, K, NP))
    for g in outs:
        assert max_rel(g[0], ref_rho) <= RHS_TOL
        for a in range(3):
            assert max_rel(g[1 + a], ref_vel[a]) <= RHS_TOL
    for g in outs[1:]:
        assert np.array_equal(outs[0], g)


def pulse(order, ne, **kw):
    cfg = workloads().gaussian_pulse(seed=1, num_elements=ne, order=order, width=1.25, sponge=1, **kw)
    cfg["IC_CENTER_X"], cfg["IC_VX_AMPLITUDE"], cfg["IC_VZ_AMPLITUDE"] = 0.3, 0.001, -0.0005
    return cfg


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6, 7])
def test_noalloc_rhs_matches_handle_rhs_twice(order):
    """Every order the kernels cover (K = 2..8: the smallest and largest
    operator blocks), with advection, LDG diffusion and sponge."""
    ne = (4, 3, 5)
    check_against_handle(pulse(order, ne), ne)


def test_noalloc_without_diffusion():
    """EVALUATE_DIFFUSION = 0: the stage kernel alone, no gradient scratch."""
    ne = (3, 4, 3)
    check_against_handle(pulse(4, ne, diffusion=False), ne)


def test_noalloc_without_sponge_null_sigma():
    """EVALUATE_SPONGE = 0 with d_sigma = NULL."""
    ne = (4, 3, 3)
    cfg = pulse(3, ne)
    cfg["EVALUATE_SPONGE"] = 0
    check_against_handle(cfg, ne)


def test_noalloc_at_the_size_limits():
    """Order 1 on 64 x 64 x 32 elements: exactly DG_NOALLOC_MAX_ELEMENTS
    elements and DG_NOALLOC_MAX_NODES node slots (8 per element)."""
    ne = (64, 64, 32)
    assert ne[0] * ne[1] * ne[2] == 131072 and ne[0] * ne[1] * ne[2] * 8 == 1048576
    cfg = workloads().gaussian_pulse(seed=2, num_elements=ne, order=1, width=0.25, sponge=2)
    check_against_handle(cfg, ne)


def test_noalloc_rejects_oversize_problem():
    m = dg()
    p = m.params_from_dict(dict(ORDER=4))
    mass = np.eye(5)
    rc = m.lib().dg_eval_rhs_noalloc(C.byref(p), mass.ctypes.data, mass.ctypes.data, 1, 1, 1, 1, 200000, None)
    assert rc == -1
    assert "too large for the static scratch" in m.lib().dg_last_error().decode()
