"""Seeded synthetic workloads, in the reference's parameter-file vocabulary.

Units are millimetres and microseconds (c0 = 1.5 mm/us for water, densities in
kg/m^3, so pressure c0^2 * drho comes out in MPa).  The reference's line solve
zeroes the mass-equation update when the row norms of M * w / rho0 drop below
its rank cutoff of 1e-6 (cppsrc/Matrix.h:320), which SI units trigger for a
1.25 mm element; the equations are invariant under this length/time rescaling,
and the cutoff never triggers in these units.

Time step (the reference fixes DT by hand; this package derives it):
    dt = CFL / ((2N + 1) * c0 * sum_a 1 / w_a)
"""
from __future__ import annotations

import math

import numpy as np

WATER = dict(C0=1.5, RHO0=1000.0, B_OVER_A=5.0, DIFF_CONST=4.3e-6)  # beta = 3.5 -> B/A = 2 (beta - 1)


def cfl_dt(cfg: dict, cfl: float = 0.5) -> float:
    N = int(cfg["ORDER"])
    inv = sum(1.0 / float(w) for w in cfg["ELEMENT_WIDTH"])
    return cfl / ((2 * N + 1) * float(cfg["C0"]) * inv)


def dof_count(cfg: dict) -> int:
    """DOFs = 4 fields (drho, u_x, u_y, u_z) at every node."""
    K = int(cfg["ORDER"]) + 1
    ne = np.prod([int(e) * int(b) for e, b in zip(cfg["NUM_ELEMENTS"], cfg.get("NUM_BLOCKS", [1, 1, 1]))])
    return int(4 * ne * K ** 3)


def gaussian_pulse(seed: int = 0, num_elements=(8, 8, 8), order: int = 3, width: float = 1.25,
                   sponge: int = 2, sigma_max: float = 0.5, periodic=(0, 0, 0), diffusion: bool = True) -> dict:
    """A single block of uniform hexes centred on the origin, water, a Gaussian
    pressure pulse of 1 MPa (sigma 1 mm) at the centre with zero velocity and
    seeded +/-1e-3 relative amplitude jitter; sponges on all six faces."""
    rng = np.random.Generator(np.random.PCG64(seed))
    amp = (1.0 / WATER["C0"] ** 2) * (1.0 + rng.uniform(-1e-3, 1e-3))
    ne = [int(v) for v in num_elements]
    cfg = dict(
        ORDER=order, NUM_ELEMENTS=ne, NUM_BLOCKS=[1, 1, 1], ELEMENT_WIDTH=[width] * 3,
        STARTING_CORNER=[-0.5 * n * width for n in ne], EVALUATE_ADVECTION=1,
        EVALUATE_DIFFUSION=int(diffusion), EVALUATE_SPONGE=1 if sponge > 0 else 0,
        BC_IS_PERIODIC=list(periodic), BC_SIGMA_MAX=sigma_max, BC_SPONGE_WIDTH=[sponge] * 6,
        IC_X_GAUSS=1, IC_Y_GAUSS=1, IC_Z_GAUSS=1, IC_DRHO_AMPLITUDE=amp, IC_VX_AMPLITUDE=0.0,
        IC_VY_AMPLITUDE=0.0, IC_VZ_AMPLITUDE=0.0, IC_SIGMA=0.5, IC_CENTER_X=0.0, IC_CENTER_Y=0.0,
        IC_CENTER_Z=0.0, **WATER)
    return cfg


def config1(seed: int = 0) -> dict:
    """Plain FP64, CPU-runnable: 8x8x8 elements on a 1 cm cube, N = 3, water,
    Gaussian pulse, 2-element sponges, CFL 0.5, 200 steps."""
    cfg = gaussian_pulse(seed)
    cfg["DT"] = cfl_dt(cfg)
    cfg["STEPS"] = 200
    return cfg


def config2(seed: int = 0) -> dict:
    """Plain FP64 at drop-in scale: 64x64x64 elements at N = 4 (32.8 M nodes)
    in 2x2x2 blocks on a 32 mm cube, water, 3-element sponges on every face but
    the source face, a 1 MHz 5-cycle Hann-windowed tone burst of 2 MPa on the
    z = 0 face with a seeded phase offset of up to 0.5 % of a cycle, CFL 0.5,
    1000 steps."""
    rng = np.random.Generator(np.random.PCG64(seed))
    phase = 2.0 * math.pi * 0.005 * rng.uniform(-1.0, 1.0)
    w = 0.5
    cfg = dict(
        ORDER=4, NUM_ELEMENTS=[32, 32, 32], NUM_BLOCKS=[2, 2, 2], ELEMENT_WIDTH=[w] * 3,
        STARTING_CORNER=[-16.0, -16.0, 0.0], EVALUATE_ADVECTION=1, EVALUATE_DIFFUSION=1,
        EVALUATE_SPONGE=1, BC_IS_PERIODIC=[0, 0, 0], BC_SIGMA_MAX=0.5, BC_SPONGE_WIDTH=[3, 3, 3, 3, 0, 3],
        IC_X_GAUSS=0, IC_Y_GAUSS=0, IC_Z_GAUSS=0, IC_DRHO_AMPLITUDE=0.0, IC_VX_AMPLITUDE=0.0,
        IC_VY_AMPLITUDE=0.0, IC_VZ_AMPLITUDE=0.0, IC_SIGMA=0.5, IC_CENTER_X=0.0, IC_CENTER_Y=0.0,
        IC_CENTER_Z=0.0, SRC_FACE=4, SRC_AMPLITUDE=2.0, SRC_FREQUENCY=1.0, SRC_CYCLES=5.0,
        SRC_PHASE=phase, SRC_RADIUS=0.0, **WATER)
    cfg["DT"] = cfl_dt(cfg)
    cfg["STEPS"] = 1000
    return cfg


def config3(seed: int = 0) -> dict:
    """Precision form of config 1: the same problem in FP32 with the
    Kahan-compensated update."""
    cfg = config1(seed)
    cfg["PRECISION"] = 32
    return cfg


FOCAL_PROBE_CONFIG1 = (0.0, 0.0, 2.5)  # on the pulse's z axis, 2.5 mm from its centre (mm)


def harmonics(t: np.ndarray, p: np.ndarray):
    """Fundamental frequency f1 (the largest non-zero DFT bin of the probe's
    pressure record, Hann-windowed) and the amplitudes |P(f1)|, |P(2 f1)| (the
    bin nearest to 2 f1).  Used as the focal-axis 2nd-harmonic measure."""
    p = np.asarray(p, dtype=np.float64)
    n = len(p)
    w = np.hanning(n)
    P = np.abs(np.fft.rfft(p * w)) * 2.0 / w.sum()
    f = np.fft.rfftfreq(n, d=float(t[1] - t[0]) if n > 1 else 1.0)
    k1 = 1 + int(np.argmax(P[1:]))
    k2 = min(len(P) - 1, int(round(2 * k1)))
    return float(f[k1]), float(P[k1]), float(P[k2])


def config4(seed: int = 0, n: int = 256, steps: int = 500, width: float = 0.25) -> list:
    """Batched form: n independent instances drawn from the seed.  Elements
    per side uniform in 4..24 (each axis independently), N uniform in
    {2, 3, 4, 5}, source amplitude log-uniform 0.1..5 MPa, centre frequency
    uniform 0.5..2 MHz, sponge thickness 2..4 elements, sound speed
    1.45..1.60 mm/us; FP32, ``steps`` RK steps each at CFL 0.5.  Each instance
    is a single block of ``width``-mm elements, zero initial state, a 5-cycle
    Hann tone burst on its z = 0 face (no sponge there) and sponges on the other
    five faces."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        ne = [int(v) for v in rng.integers(4, 25, size=3)]
        order = int(rng.integers(2, 6))
        amp = float(np.exp(rng.uniform(np.log(0.1), np.log(5.0))))
        freq = float(rng.uniform(0.5, 2.0))
        sponge = int(rng.integers(2, 5))
        c0 = float(rng.uniform(1.45, 1.60))
        cfg = dict(
            ORDER=order, NUM_ELEMENTS=ne, NUM_BLOCKS=[1, 1, 1], ELEMENT_WIDTH=[width] * 3,
            STARTING_CORNER=[-0.5 * ne[0] * width, -0.5 * ne[1] * width, 0.0], EVALUATE_ADVECTION=1,
            EVALUATE_DIFFUSION=1, EVALUATE_SPONGE=1, BC_IS_PERIODIC=[0, 0, 0], BC_SIGMA_MAX=0.5,
            BC_SPONGE_WIDTH=[sponge, sponge, sponge, sponge, 0, sponge], IC_X_GAUSS=0, IC_Y_GAUSS=0,
            IC_Z_GAUSS=0, IC_DRHO_AMPLITUDE=0.0, IC_VX_AMPLITUDE=0.0, IC_VY_AMPLITUDE=0.0,
            IC_VZ_AMPLITUDE=0.0, IC_SIGMA=0.5, IC_CENTER_X=0.0, IC_CENTER_Y=0.0, IC_CENTER_Z=0.0,
            SRC_FACE=4, SRC_AMPLITUDE=amp, SRC_FREQUENCY=freq, SRC_CYCLES=5.0, SRC_PHASE=0.0, SRC_RADIUS=0.0,
            PRECISION=32, C0=c0, RHO0=WATER["RHO0"], B_OVER_A=WATER["B_OVER_A"], DIFF_CONST=WATER["DIFF_CONST"])
        cfg["DT"] = cfl_dt(cfg)
        cfg["STEPS"] = steps
        out.append(cfg)
    return out


def scaled(cfg: dict, num_elements, num_blocks=(1, 1, 1)) -> dict:
    """The same physics on a different element count (same element width,
    domain re-centred in x and y, the z origin kept)."""
    out = dict(cfg)
    out["NUM_ELEMENTS"] = [int(v) for v in num_elements]
    out["NUM_BLOCKS"] = [int(v) for v in num_blocks]
    w = cfg["ELEMENT_WIDTH"]
    tot = [n * b for n, b in zip(out["NUM_ELEMENTS"], out["NUM_BLOCKS"])]
    corner = list(cfg["STARTING_CORNER"])
    for a in range(3):
        if not (a == 2 and cfg.get("SRC_FACE", -1) in (4, 5)):
            corner[a] = -0.5 * tot[a] * w[a]
    out["STARTING_CORNER"] = corner
    return out
