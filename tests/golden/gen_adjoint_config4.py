"""Generate the config-4 gradient fixture: the oracle's tangent-linear
gradient and FP64 central differences of the phased array's windowed loss.

Config 4: the phased array on 1024 x 1024 cells, 128 elements of 8 cells,
4000 steps; element amplitudes ~ U[0.5, 1.5] x 2e-3 and phases ~ U[0, 2 pi)
(FP32, seed CASE_SEED); loss = mean u1^2 over the 32 x 32 window centred at
(700, 512) over steps 3501-4000, on the dt schedule of the FP32 run (the
schedule the library's adjoint holds fixed, reproduced bit for bit by the
FP32 oracle). For 16 of the 256 weights (seed DIR_SEED) it records

  tlm32 : the oracle's tangent-linear model along the FP32 trajectory
          (fvo_tlm_loss: the restatement on dual numbers, values in FP32 as
          the CUDA path computes them, derivatives in double);
  tlm64 : the same along the FP64 trajectory;
  fd64  : FP64 central differences, h = 1e-4 relative (1e-4 rad for phases
          below 1 rad), on the same schedule;

and the schedule itself (adjoint_config4_schedule.npz) with the FP32 and
FP64 losses. Test infrastructure: about three hours on 8 host cores. Run
from the repo root: python tests/golden/gen_adjoint_config4.py [threads].
Each part is written as soon as it is done, and a rerun resumes.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fivonagi_gb300._abi import FV_APP_PHASED_ARRAY, FvParams  # noqa: E402
from oracle import oracle  # noqa: E402
from oracle.oracle import OracleSim, schedule_loss, tlm_loss  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "adjoint_config4.json")
SCHED = os.path.join(HERE, "adjoint_config4_schedule.npz")
CASE_SEED = 4
DIR_SEED = 16
NSTEPS = 4000
WINDOW = (700 - 16, 512 - 16, 32, 32, NSTEPS - 499, NSTEPS)  # i0, j0, ni, nj, first, last
NDIR = 16


def config4_params() -> FvParams:
    """fv_default_params(FV_APP_PHASED_ARRAY), built here without the library."""
    p = FvParams()
    p.app = FV_APP_PHASED_ARRAY
    p.cfl_even_only, p.exact, p.max_retries = 1, 1, 64
    p.cflmax, p.cflwhish = 1.0, float(np.float32(90 / 100.0))
    p.dtini = float(np.float32(0.005))
    p.nx, p.ny = 1024, 1024
    p.xmax, p.ymax = 1023.0 / 24.0, 1023.0 / 24.0
    p.beta, p.diffdelta, p.ampl, p.frec = 3.5, 5e-5, 2e-3, 1.0
    p.array_elems, p.aperture, p.center, p.ramp_periods, p.tide = 128, 1024.0, 512.0, 5.0, 0.0
    return p


def config4_case(p: FvParams):
    """(amp, phase, directions): the FP32 weights and the 16 weights checked."""
    rng = np.random.default_rng(CASE_SEED)
    amp = (rng.uniform(0.5, 1.5, p.array_elems) * p.ampl).astype(np.float32)
    ph = rng.uniform(0.0, 2 * np.pi, p.array_elems).astype(np.float32)
    dirs = np.sort(np.random.default_rng(DIR_SEED).choice(2 * p.array_elems, NDIR, replace=False)).astype(np.int32)
    return amp, ph, dirs


def fd_step(dirs, amp, ph, nelem):
    """h per direction: 1e-4 relative (1e-4 rad for phases below 1 rad)."""
    h = []
    for k in dirs:
        v = float(amp[k]) if k < nelem else float(ph[k - nelem])
        h.append(1e-4 * (abs(v) if k < nelem else max(abs(v), 1.0)))
    return h


def _save(d):
    tmp = OUT + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1)
    os.replace(tmp, OUT)


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    oracle.set_threads(threads)
    p = config4_params()
    amp, ph, dirs = config4_case(p)
    nelem = p.array_elems
    d = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            d = json.load(f)
    d.update({"case": {"app": "phased array", "nx": p.nx, "ny": p.ny, "elements": nelem, "nsteps": NSTEPS,
                       "window": list(WINDOW), "case_seed": CASE_SEED, "dir_seed": DIR_SEED,
                       "weights": "amp ~ U[0.5, 1.5] x ampl, phase ~ U[0, 2 pi), FP32, numpy default_rng(case_seed)"},
              "directions": [int(k) for k in dirs],
              "direction_names": [f"amp[{k}]" if k < nelem else f"phase[{k - nelem}]" for k in dirs]})
    if not os.path.exists(SCHED):
        t = time.time()
        o = OracleSim(p, np.float32, math="fvm")
        o.set_weights(amp, ph)
        o.init_state()
        dts, Ts = o.schedule(NSTEPS)
        o.close()
        np.savez_compressed(SCHED, dts=dts.astype(np.float32), Ts=Ts.astype(np.float32))
        print(f"schedule: {time.time() - t:.0f} s", flush=True)
    z = np.load(SCHED)
    dts, Ts = z["dts"].astype(np.float64), z["Ts"].astype(np.float64)
    for name, dtype in (("tlm32", np.float32), ("tlm64", np.float64)):
        if name in d:
            continue
        t = time.time()
        loss, g = tlm_loss(p, amp, ph, dirs, dts, Ts, WINDOW, dtype)
        d[name] = [float(x) for x in g]
        d["loss32" if dtype == np.float32 else "loss64"] = loss
        d[name + "_seconds"] = time.time() - t
        _save(d)
        print(f"{name}: {time.time() - t:.0f} s", flush=True)
    h = fd_step(dirs, amp, ph, nelem)
    d["fd64_h"] = h
    fd = d.get("fd64", [None] * NDIR)
    for r, k in enumerate(dirs):
        if fd[r] is not None:
            continue
        t = time.time()
        vals = []
        for sign in (1.0, -1.0):
            a = amp.astype(np.float64).copy()
            f = ph.astype(np.float64).copy()
            if k < nelem:
                a[k] += sign * h[r]
            else:
                f[k - nelem] += sign * h[r]
            vals.append(schedule_loss(p, a, f, dts, Ts, WINDOW, np.float64))
        fd[r] = (vals[0] - vals[1]) / (2.0 * h[r])
        d["fd64"] = fd
        _save(d)
        print(f"fd64 {d['direction_names'][r]}: {fd[r]:.10e} ({time.time() - t:.0f} s)", flush=True)
    _save(d)


if __name__ == "__main__":
    main()
