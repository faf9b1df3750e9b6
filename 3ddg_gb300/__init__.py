"""dg3d on GB300: Python binding of the C ABI in include/dg3d.h.

The product is libdg3d.so (CUDA kernels for sm_103a plus the C++ host code);
this module only loads it with ctypes and mirrors its entry points for tests,
benchmarks and scripting.  There is no fallback: if the library is missing or
a call fails, a ``DGError`` is raised.

The package directory name starts with a digit, so import it with
``importlib.import_module("3ddg_gb300")``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libdg3d.so")

DG_PRECISION_FP64 = 64
DG_PRECISION_FP32 = 32


class DGError(RuntimeError):
    pass


class DgParams(C.Structure):
    """ctypes mirror of ``dg_params`` (include/dg3d.h)."""
    _fields_ = [
        ("order", C.c_int),
        ("num_blocks", C.c_int * 3),
        ("num_elements", C.c_int * 3),
        ("elem_width", C.c_double * 3),
        ("corner", C.c_double * 3),
        ("rho0", C.c_double),
        ("c0", C.c_double),
        ("b_over_a", C.c_double),
        ("diff_const", C.c_double),
        ("eval_advect", C.c_int),
        ("eval_diff", C.c_int),
        ("eval_sponge", C.c_int),
        ("periodic", C.c_int * 3),
        ("sigma_max", C.c_double),
        ("sponge_width", C.c_int * 6),
        ("ic_gauss", C.c_int * 3),
        ("ic_drho_amp", C.c_double),
        ("ic_v_amp", C.c_double * 3),
        ("ic_sigma", C.c_double),
        ("ic_center", C.c_double * 3),
        ("precision", C.c_int),
        ("rk_exact", C.c_int),
        ("lumped_mass", C.c_int),
        ("src_face", C.c_int),
        ("src_amp", C.c_double),
        ("src_freq", C.c_double),
        ("src_cycles", C.c_double),
        ("src_phase", C.c_double),
        ("src_radius", C.c_double),
    ]


_lib = None


def lib():
    """Load libdg3d.so (built by ``build.py``); raise if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise DGError("libdg3d.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp, i, d, cp = C.c_void_p, C.c_int, C.c_double, C.c_char_p
        sig = {
            "dg_params_default": (i, [C.POINTER(DgParams)]),
            "dg_params_parse": (i, [cp, C.POINTER(DgParams), C.POINTER(d), C.POINTER(i), C.POINTER(i),
                                    C.POINTER(i), C.POINTER(i), cp]),
            "dg_create": (i, [C.POINTER(DgParams), cp, cp, C.POINTER(vp)]),
            "dg_destroy": (i, [vp]),
            "dg_step": (i, [vp, d, i]),
            "dg_synchronize": (i, [vp]),
            "dg_dims": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)]),
            "dg_get_state": (i, [vp, vp, vp]),
            "dg_set_state": (i, [vp, vp, vp]),
            "dg_set_state_async": (i, [vp, vp, vp]),
            "dg_get_state_async": (i, [vp, vp, vp]),
            "dg_step_get_state_async": (i, [vp, d, vp, vp]),
            "dg_eval_rhs": (i, [vp, vp, vp]),
            "dg_eval_rhs_noalloc": (i, [C.POINTER(DgParams), vp, vp, vp, vp, vp, vp, i, vp]),
            "dg_get_grid": (i, [vp, vp, vp]),
            "dg_time": (d, [vp]),
            "dg_write_snapshot": (i, [vp, cp, i, i]),
            "dg_launch_count": (C.c_longlong, [vp]),
            "dg_hdf5_write": (i, [cp, cp, i, C.POINTER(C.c_longlong), vp, d]),
            "dg_hdf5_read": (i, [cp, cp, i, C.POINTER(C.c_longlong), C.POINTER(i), vp, C.c_longlong,
                                 C.POINTER(i)]),
            "dg_read_snapshot": (i, [vp, cp, i]),
            "dg_probe_set": (i, [vp, i, vp]),
            "dg_probe_get": (i, [vp, vp, vp, i, C.POINTER(i)]),
            "dg_stream": (i, [vp, C.POINTER(vp)]),
            "dg_profile": (i, [vp, i]),
            "dg_kernel_stats": (i, [vp, i, C.POINTER(C.c_longlong), C.POINTER(d), C.POINTER(d), C.POINTER(d)]),
            "dg_state_device": (i, [vp, C.POINTER(vp), C.POINTER(C.c_size_t), C.POINTER(i)]),
            "dg_last_error": (cp, []),
            "dg_batch_create": (i, [i, C.POINTER(DgParams), C.POINTER(d), C.POINTER(i), cp, cp, C.POINTER(vp)]),
            "dg_batch_destroy": (i, [vp]),
            "dg_batch_step": (i, [vp, i]),
            "dg_batch_synchronize": (i, [vp]),
            "dg_batch_get_state": (i, [vp, i, vp, vp]),
            "dg_batch_info": (i, [vp, i, C.POINTER(i), C.POINTER(C.c_longlong), C.POINTER(d)]),
            "dg_batch_total_nodes": (C.c_longlong, [vp]),
            "dg_batch_autotune": (i, [vp, i, cp, C.c_size_t]),
            "dg_batch_stream": (i, [vp, C.POINTER(vp)]),
            "dg_batch_launch_count": (C.c_longlong, [vp]),
            "dg_serve_create": (i, [C.c_size_t, i, C.POINTER(vp)]),
            "dg_serve_destroy": (i, [vp]),
            "dg_serve_clock": (d, [vp]),
            "dg_serve_submit": (i, [vp, C.POINTER(DgParams), d, i, d, C.POINTER(C.c_longlong)]),
            "dg_serve_tick": (i, [vp, C.POINTER(i)]),
            "dg_serve_run": (i, [vp, d]),
            "dg_serve_result": (i, [vp, C.c_longlong, C.POINTER(d), C.POINTER(d), C.POINTER(d), vp, vp]),
            "dg_serve_stats": (i, [vp, C.POINTER(i), C.POINTER(d), C.POINTER(d), C.POINTER(d), C.POINTER(d)]),
            "dg_serve_utilization": (i, [vp, C.POINTER(d), C.POINTER(d), C.POINTER(d)]),
            "dg_write_basis_files": (i, [cp, i, i]),
            "dg_line_operators": (i, [i, i, cp, cp, vp, vp, vp, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = lib().dg_last_error().decode()
        raise DGError("%s failed (%d): %s" % (what, rc, msg))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _b(s):
    return None if s is None else os.fsencode(s)


# Parameter-file keys (the reference's names) -> dg_params fields.
def params_from_dict(cfg: dict) -> DgParams:
    p = DgParams()
    _check(lib().dg_params_default(C.byref(p)), "dg_params_default")

    def seq(key, field, conv, n):
        if key in cfg:
            vals = cfg[key]
            getattr(p, field)[:] = [conv(v) for v in vals][:n]

    if "ORDER" in cfg:
        p.order = int(cfg["ORDER"])
    seq("NUM_BLOCKS", "num_blocks", int, 3)
    seq("NUM_ELEMENTS", "num_elements", int, 3)
    seq("ELEMENT_WIDTH", "elem_width", float, 3)
    seq("STARTING_CORNER", "corner", float, 3)
    for key, field in [("RHO0", "rho0"), ("C0", "c0"), ("B_OVER_A", "b_over_a"), ("DIFF_CONST", "diff_const"),
                       ("BC_SIGMA_MAX", "sigma_max"), ("IC_DRHO_AMPLITUDE", "ic_drho_amp"),
                       ("IC_SIGMA", "ic_sigma"), ("SRC_AMPLITUDE", "src_amp"), ("SRC_FREQUENCY", "src_freq"),
                       ("SRC_CYCLES", "src_cycles"), ("SRC_PHASE", "src_phase"), ("SRC_RADIUS", "src_radius")]:
        if key in cfg:
            setattr(p, field, float(cfg[key]))
    for key, field in [("EVALUATE_ADVECTION", "eval_advect"), ("EVALUATE_DIFFUSION", "eval_diff"),
                       ("EVALUATE_SPONGE", "eval_sponge"), ("PRECISION", "precision"), ("RK_EXACT", "rk_exact"),
                       ("LUMPED_MASS", "lumped_mass"), ("SRC_FACE", "src_face")]:
        if key in cfg:
            setattr(p, field, int(cfg[key]))
    seq("BC_IS_PERIODIC", "periodic", int, 3)
    seq("BC_SPONGE_WIDTH", "sponge_width", int, 6)
    for a, k in enumerate(("IC_X_GAUSS", "IC_Y_GAUSS", "IC_Z_GAUSS")):
        if k in cfg:
            p.ic_gauss[a] = int(cfg[k])
    for a, k in enumerate(("IC_VX_AMPLITUDE", "IC_VY_AMPLITUDE", "IC_VZ_AMPLITUDE")):
        if k in cfg:
            p.ic_v_amp[a] = float(cfg[k])
    for a, k in enumerate(("IC_CENTER_X", "IC_CENTER_Y", "IC_CENTER_Z")):
        if k in cfg:
            p.ic_center[a] = float(cfg[k])
    return p


def parse_params(path: str, log_path: str | None = None):
    """Parse a reference parameter file; returns (DgParams, driver dict)."""
    p = DgParams()
    _check(lib().dg_params_default(C.byref(p)), "dg_params_default")
    dt = C.c_double(0.001)
    ns, no, ft, bf = C.c_int(1), C.c_int(1), C.c_int(1), C.c_int(1)
    _check(lib().dg_params_parse(_b(path), C.byref(p), C.byref(dt), C.byref(ns), C.byref(no), C.byref(ft),
                                 C.byref(bf), _b(log_path)), "dg_params_parse")
    return p, dict(DT=dt.value, NUM_TIME_SUBSTEPS=ns.value, NUM_OUTSTEPS=no.value, FREQ_TERMINAL=ft.value,
                   BOOL_FILE=bf.value)


class Solver:
    """One simulation on the GPU (a handle of the C ABI)."""

    def __init__(self, params, matrix_file: str | None = None, coeff_file: str | None = None):
        if isinstance(params, dict):
            params = params_from_dict(params)
        self.params = params
        h = C.c_void_p()
        _check(lib().dg_create(C.byref(params), _b(matrix_file), _b(coeff_file), C.byref(h)), "dg_create")
        self.h = h
        X, Y, Z = C.c_int(), C.c_int(), C.c_int()
        _check(lib().dg_dims(self.h, C.byref(X), C.byref(Y), C.byref(Z)), "dg_dims")
        self.dims = (X.value, Y.value, Z.value)

    h = None

    def close(self):
        if self.h:
            lib().dg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def step(self, dt: float, nsteps: int = 1):
        _check(lib().dg_step(self.h, float(dt), int(nsteps)), "dg_step")

    def synchronize(self):
        _check(lib().dg_synchronize(self.h), "dg_synchronize")

    def state(self, rho=None, vel=None):
        rho = np.empty(self.dims) if rho is None else rho
        vel = np.empty((3,) + self.dims) if vel is None else vel
        _check(lib().dg_get_state(self.h, _ptr(rho), _ptr(vel)), "dg_get_state")
        return rho, vel

    def set_state(self, rho, vel):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        _check(lib().dg_set_state(self.h, _ptr(rho), _ptr(vel)), "dg_set_state")

    def set_state_async(self, rho, vel):
        """Queue an upload from pinned, C-contiguous float64 arrays; keep them
        unchanged until ``synchronize``."""
        for a in (rho, vel):
            if not (a.flags.c_contiguous and a.dtype == np.float64):
                raise DGError("set_state_async needs C-contiguous float64 arrays")
        _check(lib().dg_set_state_async(self.h, _ptr(rho), _ptr(vel)), "dg_set_state_async")

    def step_state_async(self, dt: float, rho, vel):
        """One RK step, then a download of its result into pinned, C-contiguous
        float64 arrays (dg_step_get_state_async); they hold the state after
        ``synchronize``."""
        for a in (rho, vel):
            if not (a.flags.c_contiguous and a.dtype == np.float64):
                raise DGError("step_state_async needs C-contiguous float64 arrays")
        _check(lib().dg_step_get_state_async(self.h, float(dt), _ptr(rho), _ptr(vel)), "dg_step_get_state_async")

    def state_async(self, rho, vel):
        """Queue a download into pinned, C-contiguous float64 arrays (either may
        be None); they hold the state after ``synchronize``."""
        for a in (rho, vel):
            if a is not None and not (a.flags.c_contiguous and a.dtype == np.float64):
                raise DGError("state_async needs C-contiguous float64 arrays")
        _check(lib().dg_get_state_async(self.h, _ptr(rho), _ptr(vel)), "dg_get_state_async")

    def rhs(self):
        rho = np.empty(self.dims)
        vel = np.empty((3,) + self.dims)
        _check(lib().dg_eval_rhs(self.h, _ptr(rho), _ptr(vel)), "dg_eval_rhs")
        return rho, vel

    def grid(self):
        c = np.empty((3,) + self.dims)
        s = np.empty(self.dims)
        _check(lib().dg_get_grid(self.h, _ptr(c), _ptr(s)), "dg_get_grid")
        return c, s

    @property
    def time(self) -> float:
        return lib().dg_time(self.h)

    @property
    def launches(self) -> int:
        return lib().dg_launch_count(self.h)

    def probe_set(self, points):
        """Record the pressure at the nodes nearest to ``points`` (n x 3) after every step."""
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        self._n_probe = len(pts)
        _check(lib().dg_probe_set(self.h, len(pts), _ptr(pts)), "dg_probe_set")

    def probe_get(self):
        """(t [steps], p [steps, n]) recorded since probe_set."""
        ns = C.c_int()
        _check(lib().dg_probe_get(self.h, None, None, 0, C.byref(ns)), "dg_probe_get")
        t = np.empty(ns.value)
        p = np.empty((ns.value, self._n_probe))
        _check(lib().dg_probe_get(self.h, _ptr(t), _ptr(p), ns.value, C.byref(ns)), "dg_probe_get")
        return t, p

    @property
    def stream(self) -> int:
        """The handle's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        s = C.c_void_p()
        _check(lib().dg_stream(self.h, C.byref(s)), "dg_stream")
        return s.value or 0

    def profile(self, enable: bool = True):
        _check(lib().dg_profile(self.h, int(enable)), "dg_profile")

    def kernel_stats(self, kind: int):
        """(launches, ms, algorithmic bytes, flops) of kernel kind 0 (stage) or 1 (LDG gradient)."""
        n, ms, b, f = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        _check(lib().dg_kernel_stats(self.h, int(kind), C.byref(n), C.byref(ms), C.byref(b), C.byref(f)),
               "dg_kernel_stats")
        return n.value, ms.value, b.value, f.value

    def write_snapshot(self, folder: str, ts: int, grid: bool = False):
        _check(lib().dg_write_snapshot(self.h, _b(folder), int(ts), int(grid)), "dg_write_snapshot")

    def read_snapshot(self, folder: str, ts: int):
        """Restart: state and time from the snapshot files of time step ts."""
        _check(lib().dg_read_snapshot(self.h, _b(folder), int(ts)), "dg_read_snapshot")

    def device_state(self):
        base = (C.c_void_p * 4)()
        ns = C.c_size_t()
        ne = C.c_int()
        _check(lib().dg_state_device(self.h, base, C.byref(ns), C.byref(ne)), "dg_state_device")
        return [base[i] for i in range(4)], ns.value, ne.value


class Batch:
    """Many independent FP32 problems advanced together (dg_batch_*)."""

    def __init__(self, cfgs, matrix_file: str | None = None, coeff_file: str | None = None):
        n = len(cfgs)
        arr = (DgParams * max(n, 1))()
        dts = (C.c_double * max(n, 1))()
        steps = (C.c_int * max(n, 1))()
        for k, cfg in enumerate(cfgs):
            p = params_from_dict(cfg) if isinstance(cfg, dict) else cfg
            p.precision = DG_PRECISION_FP32
            arr[k] = p
            dts[k] = float(cfg["DT"])
            steps[k] = int(cfg.get("STEPS", 1 << 30))
        h = C.c_void_p()
        _check(lib().dg_batch_create(n, arr, dts, steps, _b(matrix_file), _b(coeff_file), C.byref(h)),
               "dg_batch_create")
        self.h = h
        self.n = n

    h = None

    def close(self):
        if self.h:
            lib().dg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def step(self, nsteps: int = 1):
        _check(lib().dg_batch_step(self.h, int(nsteps)), "dg_batch_step")

    def synchronize(self):
        _check(lib().dg_batch_synchronize(self.h), "dg_batch_synchronize")

    def info(self, i: int):
        dims = (C.c_int * 3)()
        sd = C.c_longlong()
        t = C.c_double()
        _check(lib().dg_batch_info(self.h, i, dims, C.byref(sd), C.byref(t)), "dg_batch_info")
        return tuple(dims), sd.value, t.value

    def state(self, i: int):
        dims, _, _ = self.info(i)
        rho = np.empty(dims)
        vel = np.empty((3,) + dims)
        _check(lib().dg_batch_get_state(self.h, i, _ptr(rho), _ptr(vel)), "dg_batch_get_state")
        return rho, vel

    @property
    def total_nodes(self) -> int:
        return lib().dg_batch_total_nodes(self.h)

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        _check(lib().dg_batch_stream(self.h, C.byref(s)), "dg_batch_stream")
        return s.value or 0

    @property
    def launches(self) -> int:
        return lib().dg_batch_launch_count(self.h)

    def autotune(self, trial_steps: int = 3) -> str:
        buf = C.create_string_buffer(1024)
        _check(lib().dg_batch_autotune(self.h, int(trial_steps), buf, 1024), "dg_batch_autotune")
        return buf.value.decode()


class Server:
    """Continuous-batching request loop under an HBM budget (dg_serve_*)."""

    def __init__(self, hbm_budget_bytes: int, keep_results: bool = False):
        h = C.c_void_p()
        _check(lib().dg_serve_create(int(hbm_budget_bytes), int(keep_results), C.byref(h)), "dg_serve_create")
        self.h = h
        self.dims = {}

    h = None

    def close(self):
        if self.h:
            lib().dg_serve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def clock(self) -> float:
        return lib().dg_serve_clock(self.h)

    def submit(self, cfg: dict, arrival_time: float = -1.0) -> int:
        p = params_from_dict(cfg)
        rid = C.c_longlong()
        _check(lib().dg_serve_submit(self.h, C.byref(p), float(cfg["DT"]), int(cfg["STEPS"]), float(arrival_time),
                                     C.byref(rid)), "dg_serve_submit")
        K = int(cfg["ORDER"]) + 1
        nb = cfg.get("NUM_BLOCKS", [1, 1, 1])
        self.dims[rid.value] = tuple(int(e) * int(b) * K for e, b in zip(cfg["NUM_ELEMENTS"], nb))
        return rid.value

    def tick(self) -> int:
        n = C.c_int()
        _check(lib().dg_serve_tick(self.h, C.byref(n)), "dg_serve_tick")
        return n.value

    def run(self, max_seconds: float = 0.0):
        _check(lib().dg_serve_run(self.h, float(max_seconds)), "dg_serve_run")

    def result(self, rid: int, state: bool = False):
        ta, tadm, td = C.c_double(), C.c_double(), C.c_double()
        rho = vel = None
        if state:
            dims = self.dims[rid]
            rho = np.empty(dims)
            vel = np.empty((3,) + dims)
        _check(lib().dg_serve_result(self.h, rid, C.byref(ta), C.byref(tadm), C.byref(td), _ptr(rho), _ptr(vel)),
               "dg_serve_result")
        out = {"arrival": ta.value, "admit": tadm.value, "done": td.value}
        if state:
            out["rho"], out["vel"] = rho, vel
        return out

    def stats(self):
        n, p50, p99, sps, mi = C.c_int(), C.c_double(), C.c_double(), C.c_double(), C.c_double()
        _check(lib().dg_serve_stats(self.h, C.byref(n), C.byref(p50), C.byref(p99), C.byref(sps), C.byref(mi)),
               "dg_serve_stats")
        return {"completed": n.value, "p50_s": p50.value, "p99_s": p99.value, "solves_per_s": sps.value,
                "mean_inflight": mi.value}

    def utilization(self):
        busy, span, work = C.c_double(), C.c_double(), C.c_double()
        _check(lib().dg_serve_utilization(self.h, C.byref(busy), C.byref(span), C.byref(work)),
               "dg_serve_utilization")
        return {"gpu_busy_s": busy.value, "span_s": span.value, "dof_stage_updates": work.value,
                "busy_frac": busy.value / span.value if span.value > 0 else 0.0}


def line_operators(order: int, lumped: bool = False, matrix_file=None, coeff_file=None):
    K = order + 1
    out = {k: np.empty((K, K)) for k in ("mass", "stiff", "deriv")}
    out.update({k: np.empty(K) for k in ("lift0", "liftN", "zeros")})
    _check(lib().dg_line_operators(order, int(lumped), _b(matrix_file), _b(coeff_file), _ptr(out["mass"]),
                                   _ptr(out["stiff"]), _ptr(out["deriv"]), _ptr(out["lift0"]),
                                   _ptr(out["liftN"]), _ptr(out["zeros"])), "dg_line_operators")
    return out


def hdf5_write(path: str, name: str, data, time: float = 0.0):
    """One float64 dataset + "time" in the reference's HDF5 file layout."""
    a = np.ascontiguousarray(data, dtype=np.float64)
    dims = (C.c_longlong * a.ndim)(*a.shape)
    _check(lib().dg_hdf5_write(_b(path), name.encode(), a.ndim, dims, _ptr(a), float(time)), "dg_hdf5_write")


def hdf5_read(path: str, name: str):
    """(array, type_class) of dataset ``name`` in an HDF5 file (float64 array;
    type_class 0 integer, 1 floating point).  Raises DGError whose ``code`` is
    the reference's HDF5 failure class (-1 file, -2 dataset, -3 dataspace,
    -4 datatype)."""
    L = lib()
    dims = (C.c_longlong * 32)()
    nd, cls = C.c_int(0), C.c_int(-1)
    rc = L.dg_hdf5_read(_b(path), name.encode(), 32, dims, C.byref(nd), None, 0, C.byref(cls))
    if rc == 0:
        shape = tuple(dims[i] for i in range(nd.value))
        out = np.empty(shape, dtype=np.float64)
        rc = L.dg_hdf5_read(_b(path), name.encode(), 0, None, None, _ptr(out), out.size, None)
    if rc != 0:
        err = DGError("dg_hdf5_read failed (%d): %s" % (rc, L.dg_last_error().decode()))
        err.code = rc
        raise err
    return out, cls.value


def write_basis_files(folder: str, kmax: int = 10, lumped: bool = False):
    _check(lib().dg_write_basis_files(_b(folder), kmax, int(lumped)), "dg_write_basis_files")
