"""ctypes binding of the C oracle (dg_oracle.c).  Test infrastructure only:
imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liboracle.so")


class DgoParams(C.Structure):
    _fields_ = [
        ("order", C.c_int),
        ("num_blocks", C.c_int * 3),
        ("num_elements", C.c_int * 3),
        ("elem_width", C.c_double * 3),
        ("corner", C.c_double * 3),
        ("rho0", C.c_double), ("c0", C.c_double), ("b_over_a", C.c_double), ("diff_const", C.c_double),
        ("eval_advect", C.c_int), ("eval_diff", C.c_int), ("eval_sponge", C.c_int),
        ("periodic", C.c_int * 3),
        ("sigma_max", C.c_double),
        ("sponge_width", C.c_int * 6),
        ("ic_gauss", C.c_int * 3),
        ("ic_drho_amp", C.c_double), ("ic_v_amp", C.c_double * 3), ("ic_sigma", C.c_double),
        ("ic_center", C.c_double * 3),
        ("rk_exact", C.c_int),
        ("src_face", C.c_int),
        ("src_amp", C.c_double), ("src_freq", C.c_double), ("src_cycles", C.c_double),
        ("src_phase", C.c_double), ("src_radius", C.c_double),
    ]


def build() -> str:
    """Compile liboracle.so with gcc (the oracle/Makefile recipe)."""
    os.makedirs(os.path.join(HERE, "lib"), exist_ok=True)
    src = os.path.join(HERE, "dg_oracle.c")
    if (not os.path.exists(LIB_PATH)) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "dg_oracle.h"))):
        import subprocess
        subprocess.check_call(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.dgo_create.restype = C.c_void_p
        L.dgo_create.argtypes = [C.POINTER(DgoParams), C.c_void_p, C.c_void_p, C.c_void_p]
        L.dgo_destroy.argtypes = [C.c_void_p]
        L.dgo_run.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.dgo_get_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.dgo_set_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.dgo_get_coords.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.dgo_time.restype = C.c_double
        L.dgo_time.argtypes = [C.c_void_p]
        L.dgo_rhs.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def make_params(cfg: dict) -> DgoParams:
    """cfg uses the reference's parameter names (parameters1.txt) plus
    RK_EXACT and SRC_* keys for the tone-burst source."""
    p = DgoParams()
    p.order = int(cfg["ORDER"])
    p.num_blocks[:] = [int(v) for v in cfg.get("NUM_BLOCKS", [1, 1, 1])]
    p.num_elements[:] = [int(v) for v in cfg["NUM_ELEMENTS"]]
    p.elem_width[:] = [float(v) for v in cfg["ELEMENT_WIDTH"]]
    p.corner[:] = [float(v) for v in cfg["STARTING_CORNER"]]
    p.rho0 = cfg["RHO0"]
    p.c0 = cfg["C0"]
    p.b_over_a = cfg["B_OVER_A"]
    p.diff_const = cfg["DIFF_CONST"]
    p.eval_advect = int(cfg.get("EVALUATE_ADVECTION", 0))
    p.eval_diff = int(cfg.get("EVALUATE_DIFFUSION", 0))
    p.eval_sponge = int(cfg.get("EVALUATE_SPONGE", 0))
    p.periodic[:] = [int(v) for v in cfg.get("BC_IS_PERIODIC", [0, 0, 0])]
    p.sigma_max = cfg.get("BC_SIGMA_MAX", -1.0)
    p.sponge_width[:] = [int(v) for v in cfg.get("BC_SPONGE_WIDTH", [10] * 6)]
    p.ic_gauss[:] = [int(cfg.get(k, 0)) for k in ("IC_X_GAUSS", "IC_Y_GAUSS", "IC_Z_GAUSS")]
    p.ic_drho_amp = cfg.get("IC_DRHO_AMPLITUDE", -1.0)
    p.ic_v_amp[:] = [cfg.get(k, -1.0) for k in ("IC_VX_AMPLITUDE", "IC_VY_AMPLITUDE", "IC_VZ_AMPLITUDE")]
    p.ic_sigma = cfg.get("IC_SIGMA", -1.0)
    p.ic_center[:] = [cfg.get(k, -1.0) for k in ("IC_CENTER_X", "IC_CENTER_Y", "IC_CENTER_Z")]
    p.rk_exact = int(cfg.get("RK_EXACT", 0))
    p.src_face = int(cfg.get("SRC_FACE", -1))
    p.src_amp = cfg.get("SRC_AMPLITUDE", 0.0)
    p.src_freq = cfg.get("SRC_FREQUENCY", 1.0)
    p.src_cycles = cfg.get("SRC_CYCLES", 1.0)
    p.src_phase = cfg.get("SRC_PHASE", 0.0)
    p.src_radius = cfg.get("SRC_RADIUS", 0.0)
    return p


class Oracle:
    def __init__(self, cfg: dict, M: np.ndarray, S: np.ndarray, zeros: np.ndarray):
        self.cfg = cfg
        self.K = int(cfg["ORDER"]) + 1
        nb = cfg.get("NUM_BLOCKS", [1, 1, 1])
        self.dims = tuple(int(e) * int(b) * self.K for e, b in zip(cfg["NUM_ELEMENTS"], nb))
        self._p = make_params(cfg)
        self._M = np.ascontiguousarray(M, dtype=np.float64)
        self._S = np.ascontiguousarray(S, dtype=np.float64)
        self._z = np.ascontiguousarray(zeros, dtype=np.float64)
        self.h = lib().dgo_create(C.byref(self._p), _ptr(self._M), _ptr(self._S), _ptr(self._z))
        if not self.h:
            raise RuntimeError("dgo_create failed")

    h = None

    def close(self):
        if self.h:
            lib().dgo_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def run(self, dt: float, nsteps: int):
        lib().dgo_run(self.h, float(dt), int(nsteps))

    def state(self):
        rho = np.empty(self.dims)
        vel = np.empty((3,) + self.dims)
        lib().dgo_get_state(self.h, _ptr(rho), _ptr(vel))
        return rho, vel

    def set_state(self, rho, vel):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        lib().dgo_set_state(self.h, _ptr(rho), _ptr(vel))

    def coords(self):
        c = np.empty((3,) + self.dims)
        s = np.empty(self.dims)
        lib().dgo_get_coords(self.h, _ptr(c), _ptr(s))
        return c, s

    def rhs(self):
        rho = np.empty(self.dims)
        vel = np.empty((3,) + self.dims)
        lib().dgo_rhs(self.h, _ptr(rho), _ptr(vel))
        return rho, vel

    @property
    def time(self):
        return lib().dgo_time(self.h)
