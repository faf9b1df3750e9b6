"""Generate the golden fixtures of tests/golden/ by running the reference's own
CPU solver (the FP64-promoted build oracle/_ref/ref64, compiled in place from
the reference sources by oracle/Makefile) on seeded inputs.

Run from the repository root on a machine that has the reference sources:
    make -C oracle ref && python tests/golden/make_golden.py [case ...]
(with case names, only those cases are regenerated and merged into cases.json)

Writes:
  hardcoded_coeff.txt, hardcoded_coeff2.txt, matrices.txt
      the basis inputs every case (and every test) uses, from oracle/refinputs.py;
  <case>.params.txt   the parameter file given to the reference;
  <case>.npz          drho [X][Y][Z] and vel [3][X][Y][Z] after the case's
                      steps, dt, steps, and the same from ref32 where recorded.
"""
from __future__ import annotations

import importlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import refinputs  # noqa: E402

W = importlib.import_module("3ddg_gb300.workloads")


def cases():
    out = {}
    c1 = W.config1(seed=0)
    out["c1_20"] = (c1, 20, True)
    out["c1_200"] = (c1, 200, True)

    def pulse(seed, ne, order, **kw):
        cfg = W.gaussian_pulse(seed=seed, num_elements=ne, order=order, width=1.25, sponge=1, **kw)
        cfg["IC_CENTER_X"], cfg["IC_CENTER_Y"], cfg["IC_CENTER_Z"] = 0.3, -0.2, 0.1
        cfg["IC_VX_AMPLITUDE"], cfg["IC_VZ_AMPLITUDE"] = 0.001, -0.0005
        cfg["DT"] = W.cfl_dt(cfg)
        return cfg

    out["n1_e435"] = (pulse(2, (4, 3, 5), 1), 10, False)
    out["n2_e435"] = (pulse(2, (4, 3, 5), 2), 10, False)
    out["n5_e343_periodic_xz"] = (pulse(3, (3, 4, 3), 5, periodic=(1, 0, 1)), 5, False)
    lin = pulse(4, (3, 3, 4), 4, diffusion=False)
    lin["B_OVER_A"] = 0.0
    lin["EVALUATE_SPONGE"] = 0
    out["n4_linear_nodiff"] = (lin, 5, False)
    out["n7_e222"] = (pulse(5, (2, 2, 2), 7), 3, False)

    # N = 4 with the physics of the 64^3 tone-burst workload: nonlinear flux
    # (B/A = 5), LDG diffusion and 2-element sponges on every face.
    def full4(seed, ne, centre, diff_const=None):
        cfg = W.gaussian_pulse(seed=seed, num_elements=ne, order=4, width=1.25, sponge=2)
        cfg["IC_CENTER_X"], cfg["IC_CENTER_Y"], cfg["IC_CENTER_Z"] = centre
        if diff_const is not None:
            cfg["DIFF_CONST"] = diff_const
        cfg["DT"] = W.cfl_dt(cfg)
        return cfg

    out["n4_full_e654"] = (full4(6, (6, 5, 4), (0.0, 0.0, 0.0)), 10, False)
    # off centre, with velocity and a diffusivity large enough that the LDG
    # terms move the result far above the 1e-10 bound, so every face and the
    # diffusion operator carry data
    off = full4(7, (6, 5, 4), (1.1, -0.7, 0.6), diff_const=2e-3)
    off["IC_VX_AMPLITUDE"], off["IC_VY_AMPLITUDE"], off["IC_VZ_AMPLITUDE"] = -0.0008, 0.0005, 0.001
    out["n4_full_offcentre"] = (off, 10, False)
    n6 = pulse(8, (3, 3, 3), 6)
    n6["DIFF_CONST"] = 2e-3
    out["n6_e333"] = (n6, 4, False)
    return out


def run_ref(binary, cfg, steps, basis, work):
    os.makedirs(work, exist_ok=True)
    for f in ("hardcoded_coeff.txt", "hardcoded_coeff2.txt", "matrices.txt"):
        shutil.copy(os.path.join(basis, f), work)
    p = dict(cfg)
    p.update(NUM_TIME_SUBSTEPS=steps, NUM_OUTSTEPS=1, FREQ_TERMINAL=1000000, BOOL_FILE=1)
    refinputs.write_params(os.path.join(work, "params.txt"), p)
    r = subprocess.run([binary, "params.txt", "out"], cwd=work, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s failed:\n%s\n%s" % (binary, r.stdout, r.stderr))
    rho, t = refinputs.read_raw(os.path.join(work, "out", "raw", "dRho_0_%d.bin" % steps))
    vel, _ = refinputs.read_raw(os.path.join(work, "out", "raw", "vel_0_%d.bin" % steps))
    return np.array(rho), np.array(vel), t, os.path.join(work, "params.txt")


def main(only=None):
    ref64 = os.path.join(ROOT, "oracle", "_ref", "ref64")
    ref32 = os.path.join(ROOT, "oracle", "_ref", "ref32")
    refinputs.write_coeff_files(HERE)
    refinputs.write_matrices(HERE)
    manifest = {}
    mpath = os.path.join(HERE, "cases.json")
    if only and os.path.exists(mpath):
        with open(mpath) as f:
            manifest = json.load(f)
    with tempfile.TemporaryDirectory() as tmp:
        for name, (cfg, steps, with32) in cases().items():
            if only and name not in only:
                continue
            rho, vel, t, pf = run_ref(ref64, cfg, steps, HERE, os.path.join(tmp, name))
            shutil.copy(pf, os.path.join(HERE, name + ".params.txt"))
            extra = {}
            if with32:
                r32, v32, _, _ = run_ref(ref32, cfg, steps, HERE, os.path.join(tmp, name + "_32"))
                extra = dict(rho32=r32, vel32=v32)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), rho=rho, vel=vel, time=t, dt=cfg["DT"],
                                steps=steps, **extra)
            manifest[name] = dict(steps=steps, dt=cfg["DT"], cfg={k: v for k, v in cfg.items()})
            print(name, rho.shape, "max|drho| %.6g" % np.abs(rho).max(), flush=True)
    with open(mpath, "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    # optional case names: regenerate only those and keep the other entries
    main(set(sys.argv[1:]) or None)
