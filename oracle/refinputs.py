"""Input files for running the reference's own solver as a CPU oracle.

Test infrastructure only: the product never imports this module.

The reference reads three files that it does not ship:
  * hardcoded_coeff.txt  -- per point count K = 1..KMAX: a line "n=K", a line
    of K LGL zeros on [-1, 1], a line of K LGL weights, all as 16-hex-digit IEEE
    doubles (parsed by cppsrc/Basis.cpp:133-170; mZeros[order] is the block
    with order+1 points, so the blocks must start at K = 1);
  * hardcoded_coeff2.txt -- per K: "p=K" then K rows of K hex doubles
    (cppsrc/Basis.cpp:201-236; parsed but unused by the solver);
  * matrices.txt         -- per order N: "Order=N", N+1 rows of the 1-D mass
    matrix, N+1 rows of the 1-D stiffness matrix (cppsrc/Grid.cpp:920-989).

The matrices live on the unit interval [0, 1] (the element width scales them,
cppsrc/Element.cpp:602,679,747):
    M_ij = int_0^1 l_i l_j dt        S_ij = int_0^1 l_i'(t) l_j(t) dt
with l_i the Lagrange polynomials on the LGL nodes mapped to [0, 1].  S has
this orientation because the element operator forms S*f - F with the face flux
F entering at rows 0 and N (cppsrc/Element.cpp:557-602): that is the weak form
M du/dt = int l_i' f - [l_i f*], so S_ij = int l_i' l_j.  M is the exact mass
matrix (Gauss-Legendre quadrature with N+3 points); the reference does not pin
exact versus LGL-lumped, so ``lumped=True`` writes the diagonal LGL-quadrature
mass matrix instead.

LGL nodes come from Newton iteration on x*P_N(x) - P_{N-1}(x) started from the
Chebyshev-Gauss-Lobatto points; weights are 2 / (N (N+1) P_N(x_i)^2).
"""
from __future__ import annotations

import os
import struct

import numpy as np

KMAX = 10  # point counts 1..10, i.e. orders 0..9


def lgl(K: int):
    """LGL nodes (ascending, on [-1, 1]) and weights for K points."""
    if K == 1:
        return np.array([0.0]), np.array([2.0])
    N = K - 1
    x = -np.cos(np.pi * np.arange(K) / N)
    P = np.zeros((K, K))
    for _ in range(200):
        P[:, 0] = 1.0
        P[:, 1] = x
        for k in range(2, K):
            P[:, k] = ((2 * k - 1) * x * P[:, k - 1] - (k - 1) * P[:, k - 2]) / k
        xn = x - (x * P[:, N] - P[:, N - 1]) / (K * P[:, N])
        done = np.max(np.abs(xn - x)) < 1e-16
        x = xn
        if done:
            break
    P[:, 0] = 1.0
    P[:, 1] = x
    for k in range(2, K):
        P[:, k] = ((2 * k - 1) * x * P[:, k - 1] - (k - 1) * P[:, k - 2]) / k
    w = 2.0 / (N * K * P[:, N] ** 2)
    x[0], x[-1] = -1.0, 1.0
    return x, w


def lagrange_eval(nodes: np.ndarray, t: np.ndarray):
    """Values L[q, j] = l_j(t_q) and derivatives dL[q, j] = l_j'(t_q)."""
    K = len(nodes)
    L = np.ones((len(t), K))
    dL = np.zeros((len(t), K))
    for j in range(K):
        for m in range(K):
            if m == j:
                continue
            L[:, j] *= (t - nodes[m]) / (nodes[j] - nodes[m])
        for k in range(K):
            if k == j:
                continue
            term = np.full(len(t), 1.0 / (nodes[j] - nodes[k]))
            for m in range(K):
                if m == j or m == k:
                    continue
                term *= (t - nodes[m]) / (nodes[j] - nodes[m])
            dL[:, j] += term
    return L, dL


def unit_matrices(order: int, lumped: bool = False):
    """(M, S) on [0, 1] for the given order."""
    K = order + 1
    xi, wl = lgl(K)
    t = 0.5 * (xi + 1.0)
    if lumped:
        M = np.diag(0.5 * wl)
    else:
        g, gw = np.polynomial.legendre.leggauss(K + 2)
        tq, wq = 0.5 * (g + 1.0), 0.5 * gw
        L, _ = lagrange_eval(t, tq)
        M = (L * wq[:, None]).T @ L
    g, gw = np.polynomial.legendre.leggauss(K + 2)
    tq, wq = 0.5 * (g + 1.0), 0.5 * gw
    L, dL = lagrange_eval(t, tq)
    S = (dL * wq[:, None]).T @ L
    return M, S


def hexd(v: float) -> str:
    return "%016X" % struct.unpack("<Q", struct.pack("<d", float(v)))[0]


def parse_hexd(s: str) -> float:
    return struct.unpack("<d", struct.pack("<Q", int(s, 16)))[0]


def write_coeff_files(folder: str) -> None:
    with open(os.path.join(folder, "hardcoded_coeff.txt"), "w") as f:
        for K in range(1, KMAX + 1):
            x, w = lgl(K)
            f.write("n=%d\n" % K)
            f.write(" ".join(hexd(v) for v in x) + "\n")
            f.write(" ".join(hexd(v) for v in w) + "\n")
    with open(os.path.join(folder, "hardcoded_coeff2.txt"), "w") as f:
        for K in range(1, KMAX + 1):
            x, _ = lgl(K)
            _, dL = lagrange_eval(x, x)
            f.write("p=%d\n" % K)
            for i in range(K):
                f.write(" ".join(hexd(v) for v in dL[i]) + "\n")


def write_matrices(folder: str, max_order: int = KMAX - 1, lumped: bool = False) -> None:
    with open(os.path.join(folder, "matrices.txt"), "w") as f:
        for N in range(1, max_order + 1):
            M, S = unit_matrices(N, lumped)
            f.write("Order=%d\n" % N)
            for r in M:
                f.write(" ".join(hexd(v) for v in r) + "\n")
            for r in S:
                f.write(" ".join(hexd(v) for v in r) + "\n")


def read_matrices(path: str, order: int):
    """Parse matrices.txt the way cppsrc/Grid.cpp:966-985 does."""
    K = order + 1
    rows = []
    cur = None
    with open(path) as f:
        for line in f:
            line = line.strip()
            if line.startswith("Order="):
                cur = int(line[6:])
                if cur > order:
                    break
                continue
            if cur == order and line:
                rows.append([parse_hexd(s) for s in line.split()[:K]])
    M = np.array(rows[:K])
    S = np.array(rows[K:2 * K])
    return M, S


def read_zeros(path: str, order: int):
    """LGL zeros for ``order`` from hardcoded_coeff.txt (cppsrc/Basis.cpp:133-170)."""
    with open(path) as f:
        lines = [l.strip() for l in f if l.strip()]
    blocks = [lines[i:i + 3] for i in range(0, len(lines), 3)]
    return np.array([parse_hexd(s) for s in blocks[order][1].split()])


PARAM_ORDER = [
    "NUM_TIME_SUBSTEPS", "NUM_OUTSTEPS", "FREQ_TERMINAL", "BOOL_FILE", "ORDER",
    "ELEMENT_WIDTH", "STARTING_CORNER", "DT", "C0", "DIFF_CONST", "RHO0", "B_OVER_A",
    "NUM_ELEMENTS", "NUM_BLOCKS", "EVALUATE_SPONGE", "EVALUATE_ADVECTION",
    "EVALUATE_DIFFUSION", "BC_IS_PERIODIC", "BC_SIGMA_MAX", "BC_SPONGE_WIDTH",
    "IC_X_GAUSS", "IC_Y_GAUSS", "IC_Z_GAUSS", "IC_DRHO_AMPLITUDE", "IC_VX_AMPLITUDE",
    "IC_VY_AMPLITUDE", "IC_VZ_AMPLITUDE", "IC_SIGMA", "IC_CENTER_X", "IC_CENTER_Y",
    "IC_CENTER_Z",
]


def fmt(v) -> str:
    if isinstance(v, (list, tuple, np.ndarray)):
        return " ".join(fmt(x) for x in v)
    if isinstance(v, (bool, np.bool_)):
        return "1" if v else "0"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return repr(float(v))


def write_params(path: str, params: dict) -> None:
    """Write a parameters file in the reference's "KEY = values" format
    (cppsrc/driver.cpp:139-186)."""
    with open(path, "w") as f:
        f.write("#generated parameter file\n")
        for k in PARAM_ORDER:
            if k in params:
                f.write("%s = %s\n" % (k, fmt(params[k])))


def read_raw(path: str):
    """Read a DGRAW01 file written by the reference's output stand-in."""
    with open(path, "rb") as f:
        buf = f.read()
    assert buf[:7] == b"DGRAW01", path
    nd = struct.unpack_from("<i", buf, 8)[0]
    dims = struct.unpack_from("<%dq" % nd, buf, 16)
    off = 16 + 8 * nd
    t = struct.unpack_from("<d", buf, off)[0]
    data = np.frombuffer(buf, dtype="<f8", offset=off + 8).reshape(dims)
    return data, t
