"""Benchmark: DOF-stage-updates/s of the DG right-hand side + SSP-RK3 loop.

Default workload (one GPU): 64^3 hex elements at N = 4 in 2x2x2 blocks (32.8 M
nodes, 4 fields, FP64), water, 3-element sponges, 1 MHz 5-cycle tone burst on
z = 0 (3ddg_gb300/workloads.py config2).  One bench step = one SSP-RK3 step
(3 stages) over the whole mesh.  1 DOF = one of the 4 fields at one node;
value = 4 * nodes * 3 * steps / seconds, summed over GPUs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank advances an independent replica on its own
GPU (the path does not shard here: replicas only); timing is the max over
ranks.  ``--impl reference`` times the CPU implementation of the path (the
reference's own build when it runs on this host, else the C oracle port) on the
host cores of rank 0.
"""
from __future__ import annotations

import argparse
import importlib
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
METRIC = "DOF-stage-updates/s"
UNIT = "DOF-stage-updates/s"
METRIC_NAME = "DOF-stage-updates/s FP64 vs FP32 at stated error; solves/s + p50/p99 latency"


def args_():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="RK steps of the end-to-end run (0: the same --steps as the device-timed run)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--skip-extras", action="store_true", help="skip the FP32 form and error runs")
    ap.add_argument("--elements", type=int, default=0,
                    help="profiling cases only: the config2 physics on E^3 elements in one block")
    ap.add_argument("--precision", type=int, default=64, choices=[64, 32])
    ap.add_argument("--order", type=int, default=0,
                    help="polynomial order of the device-timed workload (default: config 2's N = 4)")
    ap.add_argument("--batch-steps", type=int, default=20, help="timed RK steps of the batched form")
    ap.add_argument("--batch-instances", type=int, default=256,
                    help="problems of the batched form (config 4 has 256; fewer only for profiling)")
    ap.add_argument("--batch-tune-steps", type=int, default=2,
                    help="RK steps per autotuner trial (0: no autotuning, default tiles)")
    ap.add_argument("--serve-requests", type=int, default=500, help="requests per arrival rate (serving form)")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[15.0, 30.0, 100.0],
                    help="arrival rates (solves/s): one below and one above the server's capacity")
    ap.add_argument("--serve-baseline-rates", type=float, nargs="*", default=[15.0, 100.0])
    ap.add_argument("--serve-baseline-requests", type=int, default=24,
                    help="first requests of a trace served one at a time through the FP64 plain path")
    ap.add_argument("--serve-only", action="store_true",
                    help="run only the serving form (a rate sweep) and print its JSON object")
    return ap.parse_args()


# ---------------------------------------------------------------- distributed
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as tdist
            backend = "nccl" if self._cuda() else "gloo"
            if backend == "nccl":
                import torch
                torch.cuda.set_device(self.local_rank)
            tdist.init_process_group(backend=backend)
            self.pg = tdist

    @staticmethod
    def _cuda():
        try:
            import torch
            return torch.cuda.is_available()
        except Exception:
            return False

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        return reduce_max(self.pg, x)

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def reduce_max(pg, x: float) -> float:
    """Max of a float over all ranks (identity without a process group)."""
    if pg is None:
        return float(x)
    import torch
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- helpers
# Orders N whose FP64 stage / gradient kernels use even-odd line owners (K = N + 1;
# eo_lines and eo_grad_lines in 3ddg_gb300/csrc/dg_kernels.cuh), for the kernel labels.
EO_STAGE_ORDERS = (1, 2, 4)
EO_GRAD_ORDERS = (1, 2, 3, 4)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


FP64_PEAK_TFLOPS = 1.19  # FP64 FMA throughput measured on a GB300 (8 independent DFMA chains per thread, all SMs)

# Algorithmic HBM bytes per DOF-stage-update of the FP32 increment form with diffusion (4 DOFs per
# node): stage kernel (11 + 15 + 23) / 3 values of 4 B per node over the three stages (input u, d,
# G, compensation in; d or u', compensation out), gradient kernel (4 + 5 + 5) / 3 values; 84 B per
# node-stage.
FP32_BYTES_PER_DOF_STAGE = 84.0 / 4


def hbm_roofline(value):
    """Whole-job HBM fraction of an FP32 form's throughput from its algorithmic bytes."""
    peak, kind = measured_peaks()
    gbs = value * FP32_BYTES_PER_DOF_STAGE / 1e9
    return {"bound": "hbm", "algorithmic_bytes_per_dof_stage": FP32_BYTES_PER_DOF_STAGE, "achieved_gbs": gbs,
            "peak_gbs": peak, "frac": gbs / peak, "peak_source": kind}


def profiled_traffic(kind: str):
    """Per-launch DRAM traffic of the dominant kernel from the committed ncu
    summary (profiles/<kernel>_<workload>.md, line 'TRAFFIC_BYTES_PER_LAUNCH =')."""
    path = os.path.join(ROOT, "profiles", "stage_kernel_%s_config2.md" % kind)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for ln in f:
            if ln.strip().startswith("TRAFFIC_BYTES_PER_LAUNCH"):
                try:
                    return float(ln.split("=")[1].split()[0])
                except Exception:
                    return None
    return None


def pressure(cfg, drho):
    c0, r0, ba = cfg["C0"], cfg["RHO0"], cfg["B_OVER_A"]
    return c0 * c0 * (drho + ba / (2.0 * r0) * drho * drho)


def _oracle_sample_worker(args):
    """One CPU process of the baseline: the C oracle (or the reference's own
    build) advancing a sub-mesh of the workload for about ``seconds``."""
    cfg, seconds, max_steps, ref_bin, workdir = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    W = importlib.import_module("3ddg_gb300.workloads")
    nodes = W.dof_count(cfg) // 4
    if ref_bin:
        import refinputs
        os.makedirs(workdir, exist_ok=True)
        refinputs.write_coeff_files(workdir)
        refinputs.write_matrices(workdir)
        def timed(n):
            p = dict(cfg)
            p.update(NUM_TIME_SUBSTEPS=n, NUM_OUTSTEPS=1, FREQ_TERMINAL=10 ** 9, BOOL_FILE=0)
            refinputs.write_params(os.path.join(workdir, "p.txt"), p)
            t0 = time.perf_counter()
            subprocess.run([ref_bin, "p.txt", "out"], cwd=workdir, capture_output=True, check=True)
            return time.perf_counter() - t0

        # the program's set-up (mesh, IC, files) is timed alone and subtracted
        setup = timed(0)
        one = max(timed(1) - setup, 1e-3)
        n = int(max(1, min(max_steps, seconds / one)))
        return n, max(timed(n) - setup, 1e-6), nodes
    import pyoracle
    import refinputs
    M, S = refinputs.unit_matrices(int(cfg["ORDER"]))
    z, _ = refinputs.lgl(int(cfg["ORDER"]) + 1)
    o = pyoracle.Oracle(cfg, M, S, z)
    o.run(cfg["DT"], 1)  # first step outside the timing (allocation, first touch)
    steps_done, t0 = 0, time.perf_counter()
    while steps_done < max_steps and time.perf_counter() - t0 < seconds:
        o.run(cfg["DT"], 1)
        steps_done += 1
    return steps_done, time.perf_counter() - t0, nodes


def reference_binary():
    """The reference's own FP64 build, if it exists and runs on this host."""
    b = os.path.join(ROOT, "oracle", "_ref", "ref64")
    if not os.path.exists(b):
        return None
    try:
        r = subprocess.run([b], capture_output=True, timeout=20)
        return b if r.returncode in (0, 1) else None
    except Exception:
        return None


def cpu_sample_cfg(cfg, ne=(12, 12, 12)):
    W = importlib.import_module("3ddg_gb300.workloads")
    s = W.scaled(cfg, ne)
    s.pop("PRECISION", None)
    return s


def cpu_baseline(cfg, processes: int, seconds: float, max_steps: int = 10 ** 6):
    sample = cpu_sample_cfg(cfg)
    ref_bin = reference_binary()
    ctx = mp.get_context("spawn")
    jobs = [(sample, seconds, max_steps, ref_bin, "/tmp/dg3d_cpu_baseline_%d_%d" % (os.getpid(), i))
            for i in range(processes)]
    with ctx.Pool(processes) as pool:
        res = pool.map(_oracle_sample_worker, jobs)
    rate = sum(4 * nodes * 3 * steps / dt for steps, dt, nodes in res)
    steps = min(r[0] for r in res)
    ne = sample["NUM_ELEMENTS"]
    desc = ("%d process(es), each %dx%dx%d elements at N=%d of the same physics (%d nodes), %d+ RK steps in ~%.0f s"
            % (processes, ne[0], ne[1], ne[2], sample["ORDER"], res[0][2], steps, seconds))
    return {"value": rate, "unit": UNIT, "cores": processes, "kind": "reference" if ref_bin else "port",
            "sample": desc}


# ---------------------------------------------------------------- our arm
def run_ours(a, dist: Dist):
    import torch
    dg = importlib.import_module("3ddg_gb300")
    W = importlib.import_module("3ddg_gb300.workloads")
    dev = dist.local_rank if dist.world > 1 else 0
    torch.cuda.set_device(dev)
    cfg = W.config2(seed=dist.rank)
    if a.elements:
        cfg = W.scaled(cfg, (a.elements,) * 3)
    if a.order:
        cfg["ORDER"] = a.order
        cfg["DT"] = W.cfl_dt(cfg)
    if a.precision == 32:
        cfg["PRECISION"] = 32
    dt = cfg["DT"]
    nodes = W.dof_count(cfg) // 4
    s = dg.Solver(cfg)
    stream = torch.cuda.ExternalStream(s.stream)

    s.step(dt, a.warmup)
    s.synchronize()
    dist.barrier()
    torch.cuda.synchronize()
    l0 = s.launches
    s.profile(True)
    clocks = ClockSampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(dev)).split(",")[0])
                          if os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].isdigit() else dev)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.step(dt, a.steps)
    e1.record(stream)
    e1.synchronize()
    ck = clocks.stop()
    torch.cuda.synchronize()
    dist.barrier()
    ms = e0.elapsed_time(e1)
    launches = s.launches - l0
    st_n, st_ms, st_b, st_f = s.kernel_stats(0)
    gr_n, gr_ms, gr_b, gr_f = s.kernel_stats(1)
    s.profile(False)
    ms_max = dist.max(ms)
    dofs = 4 * nodes * 3 * a.steps
    value = dist.world * dofs / (ms_max / 1e3)

    # e2e through the public API with pinned host buffers: every step copies
    # its input state host->device and its result device->host.  The headline
    # uses the asynchronous calls (copies on the copy engines, overlapping the
    # neighbouring steps' compute); the synchronous calls are timed too.
    X, Y, Z = s.dims
    rho_t = torch.empty((X, Y, Z), dtype=torch.float64, pin_memory=True)
    vel_t = torch.empty((3, X, Y, Z), dtype=torch.float64, pin_memory=True)
    rho_o = torch.empty((X, Y, Z), dtype=torch.float64, pin_memory=True)
    vel_o = torch.empty((3, X, Y, Z), dtype=torch.float64, pin_memory=True)
    rho, vel, rho_out, vel_out = rho_t.numpy(), vel_t.numpy(), rho_o.numpy(), vel_o.numpy()
    s.state(rho, vel)
    ne2e = max(1, a.e2e_steps if a.e2e_steps > 0 else a.steps)
    dist.barrier()
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(ne2e):
        s.set_state_async(rho, vel)
        s.step_state_async(dt, rho_out, vel_out)
    s.synchronize()  # every copy has landed in host memory
    f1.record(stream)
    f1.synchronize()
    e2e_ms = dist.max(f0.elapsed_time(f1))
    e2e_value = dist.world * 4 * nodes * 3 * ne2e / (e2e_ms / 1e3)
    # the same loop with the step and the download as separate calls
    dist.barrier()
    torch.cuda.synchronize()
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(stream)
    for _ in range(ne2e):
        s.set_state_async(rho, vel)
        s.step(dt, 1)
        s.state_async(rho_out, vel_out)
    s.synchronize()
    h1.record(stream)
    h1.synchronize()
    sep_ms = dist.max(h0.elapsed_time(h1))
    dist.barrier()
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(ne2e):
        s.set_state(rho, vel)
        s.step(dt, 1)
        s.state(rho_out, vel_out)
    g1.record(stream)
    g1.synchronize()
    sync_ms = dist.max(g0.elapsed_time(g1))
    step_bytes = 4 * nodes * 8
    s.close()

    extras = {}
    if not a.skip_extras and dist.rank == 0:
        extras = precision_form(a, cfg, dg, W, torch)
        extras["batched_form"] = batched_form(a, dg, W, torch)
        if a.serve_requests > 0:
            extras["serving_form"] = serving_form(a, dg, W)

    if dist.rank != 0:
        return None
    peak, peak_kind = measured_peaks()
    kind = "fp64"
    fp64 = cfg.get("PRECISION", 64) == 64
    ctype = "double" if fp64 else "float"
    ne_g = [cfg["NUM_ELEMENTS"][i] * cfg["NUM_BLOCKS"][i] for i in range(3)]
    nb = cfg["NUM_BLOCKS"]
    buf_gb = 4 * nodes * (8 if fp64 else 4) / 1e9
    workload = ("%s: %dx%dx%d hex elements N=%d in %dx%dx%d blocks, %s, water, tone burst, adv+LDG diffusion+sponge"
                % ("config2" if not (a.elements or a.order) else "config2 physics, resized", ne_g[0], ne_g[1], ne_g[2],
                   cfg["ORDER"], nb[0], nb[1], nb[2], "FP64" if fp64 else "FP32"))
    ach = (st_b / st_n) / (st_ms / st_n / 1e3) / 1e9 if st_n else None
    traffic = profiled_traffic(kind)
    roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": (ach / peak) if ach else None,
            "traffic": traffic, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s",
            "kernel": (("stage_kernel<double,%d,DIFF,2,EO> (fluxes read, even-odd line owners)" % (cfg["ORDER"] + 1)
                        if cfg["ORDER"] in EO_STAGE_ORDERS
                        else "stage_kernel<double,%d,DIFF,2> (fluxes read, per-node line sums)" % (cfg["ORDER"] + 1))
                       if fp64 else "incr_stage_kernel<float,%d,DIFF>" % (cfg["ORDER"] + 1)),
            "algorithmic_bytes_per_launch": st_b / st_n if st_n else None,
            "traffic_note": ("above the algorithmic bytes by the volume-flux buffers (4 values written and 4 read "
                             "per node, 64 B): HBM traded for the FP64 work of evaluating each face neighbour's "
                             "flux a second time" if fp64 else None),
            "mean_launch_ms": st_ms / st_n if st_n else None,
            "fp64_pipe": {"achieved_tflops": (st_f / st_n) / (st_ms / st_n / 1e3) / 1e12 if st_n else None,
                          "peak_tflops": FP64_PEAK_TFLOPS,
                          "frac": ((st_f / st_n) / (st_ms / st_n / 1e3) / 1e12) / FP64_PEAK_TFLOPS if st_n else None,
                          "note": "the FP64 path is bound by the FP64 pipe (1.19 TFLOP/s measured), not HBM; "
                                  "flops counted by the direct formula (K (K + 2) per line), which the even-odd "
                                  "line owners execute with about 22 % fewer FP64 instructions"},
            "share_of_step": st_ms / ms if ms else None,
            "gradient_kernel": {"name": ("ldg_gradient_eo_kernel<%d>" % (cfg["ORDER"] + 1)
                                         if fp64 and cfg["ORDER"] in EO_GRAD_ORDERS else
                                         ("ldg_gradient_kernel<double,%d>" if fp64 else "ldg_gradient_kernel<float,%d>")
                                         % (cfg["ORDER"] + 1)),
                                "launches": gr_n, "mean_launch_ms": gr_ms / gr_n if gr_n else None,
                                "achieved_gbs": (gr_b / gr_n) / (gr_ms / gr_n / 1e3) / 1e9 if gr_n else None}}
    line = {
        "metric": METRIC_NAME, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if fp64 else "f32", "data": "synthetic (seeded tone burst, no IC)",
        "config": {"workload": workload, "nodes": nodes, "dofs": 4 * nodes,
                   "parallelism": "replicas" if dist.world > 1 else "single GPU",
                   "l2": "inputs %s than L2 (state %.3g GB per buffer)" % ("larger" if buf_gb > 0.129 else "smaller",
                                                                          buf_gb), "dt_us": dt},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": step_bytes, "d2h_bytes_per_step": step_bytes,
                "steps": ne2e, "ms_per_step": e2e_ms / ne2e,
                "mode": "dg_set_state_async + dg_step_get_state_async per step from/to pinned host buffers, "
                        "timed from the first upload to the last download landing in host memory",
                "separate_calls": {"value": dist.world * 4 * nodes * 3 * ne2e / (sep_ms / 1e3),
                                   "ms_per_step": sep_ms / ne2e,
                                   "mode": "dg_set_state_async + dg_step + dg_get_state_async per step"},
                "sync_calls": {"value": dist.world * 4 * nodes * 3 * ne2e / (sync_ms / 1e3),
                               "ms_per_step": sync_ms / ne2e,
                               "mode": "dg_set_state + dg_step + dg_get_state (synchronous) per step"}},
        "gpu_launches": launches,
        "clocks": ck,
        "roofline": roof,
    }
    line.update(extras)
    return line


def precision_form(a, cfg, dg, W, torch):
    """The FP32 chosen form on the same workload, and its error against the
    FP64 path on config 3 (= config 1 in FP32, 200 steps)."""
    out = {}
    cfg32 = dict(cfg)
    cfg32["PRECISION"] = 32
    s = dg.Solver(cfg32)
    stream = torch.cuda.ExternalStream(s.stream)
    s.step(cfg["DT"], a.warmup)
    s.synchronize()
    s.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.step(cfg["DT"], a.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    st_n, st_ms, st_b, _ = s.kernel_stats(0)
    s.profile(False)
    s.close()
    nodes = W.dof_count(cfg) // 4
    v32 = 4 * nodes * 3 * a.steps / (ms / 1e3)
    peak, _ = measured_peaks()
    ach = (st_b / st_n) / (st_ms / st_n / 1e3) / 1e9 if st_n else None
    c1 = W.config1(seed=0)
    c3 = W.config3(seed=0)
    s64, s32 = dg.Solver(c1), dg.Solver(c3)
    for s_ in (s64, s32):
        s_.probe_set([W.FOCAL_PROBE_CONFIG1])
        s_.step(c1["DT"], c1["STEPS"])
    r64, _ = s64.state()
    r32, _ = s32.state()
    t64, pr64 = s64.probe_get()
    _, pr32 = s32.probe_get()
    s64.close()
    s32.close()
    p64, p32 = pressure(c1, r64), pressure(c1, r32)
    f1, a1, h2_64 = W.harmonics(t64, pr64[:, 0])
    _, _, h2_32 = W.harmonics(t64, pr32[:, 0])
    out["fp32_form"] = {
        "value": v32, "unit": UNIT, "ms_per_step": ms / a.steps, "speedup_vs_fp64": None,
        "stage_kernel_hbm_gbs": ach, "stage_kernel_hbm_frac": ach / peak if ach else None,
        "error_vs_fp64_config3": {"l2_rel_pressure": float(np.linalg.norm(p32 - p64) / np.linalg.norm(p64)),
                                  "linf_rel_pressure": float(np.max(np.abs(p32 - p64)) / np.max(np.abs(p64))),
                                  "second_harmonic_rel": abs(h2_32 - h2_64) / h2_64 if h2_64 else None,
                                  "focal_probe_mm": list(W.FOCAL_PROBE_CONFIG1), "fundamental_mhz": f1,
                                  "second_harmonic_fp64": h2_64, "fundamental_amp_fp64": a1,
                                  "steps": c1["STEPS"]},
    }
    return out


def batched_form(a, dg, W, torch):
    """Config 4: 256 uneven FP32 problems (N in 2..5) advanced together by
    persistent kernels per order, as parallel branches of a CUDA graph;
    autotuned tiles."""
    cfgs = W.config4(seed=0, n=a.batch_instances)
    steps = max(1, min(a.batch_steps, 400))
    with dg.Batch(cfgs) as b:
        nodes = b.total_nodes
        t0 = time.perf_counter()
        tune = b.autotune(a.batch_tune_steps) if a.batch_tune_steps > 0 else "default tiles"
        tune_s = time.perf_counter() - t0
        stream = torch.cuda.ExternalStream(b.stream)
        b.step(a.warmup)
        b.synchronize()
        l0 = b.launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        launches = b.launches - l0
        # error of the FP32 batch against the FP64 plain path, one problem per order
        err = {}
        picks = {}
        for i, c in enumerate(cfgs):
            picks.setdefault(c["ORDER"], i)
        for order, i in sorted(picks.items()):
            _, done, _ = b.info(i)
            r32, _ = b.state(i)
            c64 = dict(cfgs[i], PRECISION=64)
            with dg.Solver(c64) as s64:
                s64.step(c64["DT"], int(done))
                r64, _ = s64.state()
            p32, p64 = pressure(c64, r32), pressure(c64, r64)
            err["N=%d" % order] = {"problem": i, "steps": int(done),
                                   "l2_rel_pressure": float(np.linalg.norm(p32 - p64) / np.linalg.norm(p64)),
                                   "linf_rel_pressure": float(np.max(np.abs(p32 - p64)) / np.max(np.abs(p64)))}
    return {"value": 4 * nodes * 3 * steps / (ms / 1e3), "unit": UNIT, "problems": len(cfgs), "nodes": nodes,
            "orders": sorted({c["ORDER"] for c in cfgs}), "steps": steps, "ms_per_step": ms / steps,
            "error_vs_fp64": err, "roofline": hbm_roofline(4 * nodes * 3 * steps / (ms / 1e3)),
            "autotune": tune, "autotune_s": tune_s, "graph_launches_per_step": launches / steps,
            "workload": "config4: %d instances, elements 4..24 per axis, N 2..5, FP32 Kahan, tone burst, sponge"
                        % len(cfgs)}


def serving_trace(rate: float, n: int, seed: int, W):
    """Open-loop Poisson arrivals at ``rate`` solves/s; each request drawn from
    the batched-form distribution with steps uniform in 100..2000."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cfgs = W.config4(seed=seed + 1000, n=n)
    t = 0.0
    arrivals = []
    for c in cfgs:
        t += rng.exponential(1.0 / rate)
        arrivals.append(t)
        c["STEPS"] = int(rng.integers(100, 2001))
    return cfgs, arrivals


def serving_form(a, dg, W):
    """Config 5: continuous batching under a 150 GB HBM budget, swept over
    arrival rates, against one-solve-at-a-time service through the FP64 plain
    path on the same trace."""
    out = {"budget_gb": 150, "requests_per_rate": a.serve_requests, "rates": []}
    for k, rate in enumerate(a.serve_rates):
        cfgs, arr = serving_trace(rate, a.serve_requests, 40 + k, W)
        with dg.Server(150 << 30) as srv:
            t0 = srv.clock + 0.05
            for c, ta in zip(cfgs, arr):
                srv.submit(c, arrival_time=t0 + ta)
            srv.run(max_seconds=900)
            st = srv.stats()
            u = srv.utilization()
        work = sum(W.dof_count(c) * 3 * c["STEPS"] for c in cfgs)
        row = {"rate_per_s": rate, "requests": len(cfgs),
               # the seeded Poisson trace's own rate: (n - 1) / (last arrival - first arrival)
               "arrival_rate_realized": (len(arr) - 1) / max(1e-9, arr[-1] - arr[0]),
               "p50_s": st["p50_s"], "p99_s": st["p99_s"],
               "solves_per_s": st["solves_per_s"], "mean_inflight": st["mean_inflight"],
               "completed": st["completed"], "dof_stage_updates": work,
               # served throughput over the trace's span (first arrival to last completion)
               "dof_stage_updates_per_s": work / max(1e-9, u["span_s"]),
               # device time inside RK steps over the span, and the throughput over that time
               "gpu_busy_frac": u["busy_frac"],
               "dof_stage_updates_per_gpu_busy_s": u["dof_stage_updates"] / max(1e-9, u["gpu_busy_s"])}
        row["hbm_frac"] = hbm_roofline(row["dof_stage_updates_per_s"])["frac"]
        if rate in a.serve_baseline_rates:
            nb = min(len(cfgs), a.serve_baseline_requests)
            bwork = sum(W.dof_count(c) * 3 * c["STEPS"] for c in cfgs[:nb])
            lat, span0, span1, prev_done = [], None, 0.0, 0.0
            start = time.perf_counter()
            for c, ta in zip(cfgs[:nb], arr[:nb]):
                c64 = dict(c)
                c64["PRECISION"] = 64
                begin = max(ta, prev_done)
                now = time.perf_counter() - start
                if begin > now:
                    time.sleep(begin - now)
                with dg.Solver(c64) as s:
                    s.step(c64["DT"], c64["STEPS"])
                    s.synchronize()
                prev_done = time.perf_counter() - start
                lat.append(prev_done - ta)
            lat.sort()
            span = max(1e-9, prev_done - arr[0])
            row["fp64_one_at_a_time"] = {"requests": nb, "p50_s": float(np.percentile(lat, 50)),
                                         "p99_s": float(np.percentile(lat, 99)),
                                         "solves_per_s": len(lat) / span, "dof_stage_updates_per_s": bwork / span}
        out["rates"].append(row)
    # error of served results against the FP64 plain path: one request per order of the first
    # trace, served together (untimed, results kept) and each solved alone in FP64
    cfgs, _ = serving_trace(a.serve_rates[0], a.serve_requests, 40, W)
    picks = {}
    for c in cfgs:
        picks.setdefault(c["ORDER"], c)
    err = {}
    with dg.Server(150 << 30, keep_results=True) as srv:
        rids = {order: srv.submit(c) for order, c in sorted(picks.items())}
        srv.run(max_seconds=600)
        for order, rid in rids.items():
            c64 = dict(picks[order], PRECISION=64)
            r32 = srv.result(rid, state=True)["rho"]
            with dg.Solver(c64) as s64:
                s64.step(c64["DT"], c64["STEPS"])
                r64, _ = s64.state()
            p32, p64 = pressure(c64, r32), pressure(c64, r64)
            err["N=%d" % order] = {"steps": c64["STEPS"],
                                   "l2_rel_pressure": float(np.linalg.norm(p32 - p64) / np.linalg.norm(p64)),
                                   "linf_rel_pressure": float(np.max(np.abs(p32 - p64)) / np.max(np.abs(p64)))}
    out["error_vs_fp64"] = err
    return out


def run_reference(a, dist: Dist):
    if dist.rank != 0:
        return None
    W = importlib.import_module("3ddg_gb300.workloads")
    cfg = W.config2(seed=0)
    procs = os.cpu_count() or 1
    # warm-up + timed steps of the sample, all host cores in parallel
    base = cpu_baseline(cfg, procs, seconds=max(2.0, 0.5 * (a.steps + a.warmup)), max_steps=a.steps)
    value = base["value"]
    line = {
        "metric": METRIC_NAME, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded tone burst, no IC)",
        "config": {"workload": "config2: 64x64x64 hex elements N=4 in 2x2x2 blocks, FP64, water, tone burst, "
                               "adv+LDG diffusion+sponge", "sample": base["sample"]},
        "impl": "reference",
        "cpu_baseline": base,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return line


def main():
    a = args_()
    dist = Dist()
    try:
        if a.impl == "reference":
            line = run_reference(a, dist)
        elif a.serve_only:
            line = None
            if dist.rank == 0:
                line = {"serving_form": serving_form(a, importlib.import_module("3ddg_gb300"),
                                                     importlib.import_module("3ddg_gb300.workloads"))}
        else:
            line = run_ours(a, dist)
            if line is not None and dist.rank == 0 and dist.world == 1 and a.cpu_seconds > 0:
                W = importlib.import_module("3ddg_gb300.workloads")
                line["cpu_baseline"] = cpu_baseline(W.config2(seed=0), 1, a.cpu_seconds)
                fp32 = line.get("fp32_form")
                if fp32:
                    fp32["speedup_vs_fp64"] = fp32["value"] / line["value"]
                bf = line.get("batched_form")
                if bf:
                    bf["speedup_vs_fp64_plain"] = bf["value"] / line["value"]
                sf = line.get("serving_form")
                if sf and sf["rates"]:
                    # the highest arrival rate saturates the GPU: served throughput there
                    top = max(sf["rates"], key=lambda r: r["rate_per_s"])
                    sf["saturated_dof_stage_updates_per_s"] = top["dof_stage_updates_per_s"]
                    sf["saturated_vs_fp64_plain"] = top["dof_stage_updates_per_s"] / line["value"]
                    sf["capacity_solves_per_s"] = top["solves_per_s"]
                    # highest tested rate the server keeps up with (completions keep pace with arrivals)
                    kept = [r["rate_per_s"] for r in sf["rates"]
                            if r["solves_per_s"] >= 0.95 * r["arrival_rate_realized"]]
                    sf["sustained_rate_per_s"] = max(kept) if kept else None
                    if bf:
                        sf["saturated_busy_vs_batched"] = top["dof_stage_updates_per_gpu_busy_s"] / bf["value"]
                        sf["saturated_span_vs_batched"] = top["dof_stage_updates_per_s"] / bf["value"]
        if line is not None:
            print(json.dumps(line), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
