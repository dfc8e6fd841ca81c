"""Generate the config-5 gradient fixture: FP64 central differences of one
design's windowed loss, the FP64 oracle gradient the batched adjoint's
per-design error is measured against.

Config 5: designs of the phased array on 2048 x 1024 cells, 128 elements
of 8 cells, 6000 steps, beta 3.5, dissipation 5e-5. Design d (as bench.py's
designs workload builds it): element amplitudes ~ U[0.5, 1.5] x 2e-3 and
phases ~ U[0, 2 pi) (FP32, numpy default_rng(1000 + d)); loss = mean u1^2
over the 32 x 32 window centred on target d of a seeded permutation
(default_rng(0)) of an 8 x 8 grid of focal points in the right half, over
steps 5501-6000, on the dt schedule of the FP32 run. For design DESIGN and
NDIR of its 256 weights (seed DIR_SEED) it records

  fd64 : FP64 central differences, h = 1e-4 relative (1e-4 rad for phases
         below 1 rad), on that schedule;

and the schedule itself (adjoint_config5_schedule.npz) with the FP32 loss.
Test infrastructure: about two hours on 8 host cores. Run from the repo
root: python tests/golden/gen_adjoint_config5.py [threads]. Each part is
written as soon as it is done, and a rerun resumes.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from oracle.oracle import OracleSim, schedule_loss  # noqa: E402
from tests.golden.gen_adjoint_config4 import config4_params, fd_step  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "adjoint_config5.json")
SCHED = os.path.join(HERE, "adjoint_config5_schedule.npz")
NSTEPS = 6000
DESIGN = 0
TARGET_SEED = 0   # bench.py --seed 0: the focal targets' permutation
DESIGN_SEED = 1000  # design d's weights: default_rng(DESIGN_SEED + d)
DIR_SEED = 5
NDIR = 4


def config5_params():
    """The phased array's defaults (fv_default_params) on 2048 x 1024."""
    p = config4_params()
    p.nx, p.ny = 2048, 1024
    p.xmax, p.ymax = 2047.0 / 24.0, 1023.0 / 24.0
    p.center = 512.0
    return p


def config5_case(p, d: int = DESIGN):
    """(amp, phase, window, directions) of design d, as bench.py builds it."""
    rng = np.random.default_rng(TARGET_SEED)
    targets = [(1024 + 128 * (k % 8) + 64, 128 * (k // 8) + 64) for k in rng.permutation(64)]
    wr = np.random.default_rng(DESIGN_SEED + d)
    amp = (wr.uniform(0.5, 1.5, p.array_elems) * p.ampl).astype(np.float32)
    ph = wr.uniform(0.0, 2 * np.pi, p.array_elems).astype(np.float32)
    i, j = (int(x) for x in targets[d])
    window = (i - 16, j - 16, 32, 32, max(1, NSTEPS - 499), NSTEPS)
    dirs = np.sort(np.random.default_rng(DIR_SEED).choice(2 * p.array_elems, NDIR, replace=False)).astype(np.int32)
    return amp, ph, window, dirs


def _save(d):
    tmp = OUT + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1)
    os.replace(tmp, OUT)


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    oracle.set_threads(threads)
    p = config5_params()
    amp, ph, window, dirs = config5_case(p)
    nelem = p.array_elems
    d = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            d = json.load(f)
    d.update({"case": {"app": "phased array", "nx": p.nx, "ny": p.ny, "elements": nelem, "nsteps": NSTEPS,
                       "design": DESIGN, "window": list(window), "target_seed": TARGET_SEED,
                       "design_seed": DESIGN_SEED + DESIGN, "dir_seed": DIR_SEED,
                       "weights": "amp ~ U[0.5, 1.5] x ampl, phase ~ U[0, 2 pi), FP32, numpy default_rng(design_seed)"},
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
    if "loss32" not in d:
        d["loss32"] = schedule_loss(p, amp.astype(np.float64), ph.astype(np.float64), dts, Ts, window, np.float32)
        _save(d)
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
            vals.append(schedule_loss(p, a, f, dts, Ts, window, np.float64))
        fd[r] = (vals[0] - vals[1]) / (2.0 * h[r])
        d["fd64"] = fd
        _save(d)
        print(f"fd64 {d['direction_names'][r]}: {fd[r]:.10e} ({time.time() - t:.0f} s)", flush=True)
    _save(d)


if __name__ == "__main__":
    main()
