"""Generate tests/golden/ fixtures from the reference's own headers.

Runs the host build of the reference (oracle/_ref/libfvref.so, made by
oracle/Makefile from the reference tree) on small seeded cases of every app,
in FP32 and FP64, and stores what it produced:

  golden_small.npz   full output grids of 32x16 cases: the init hook, each
                     stage of one step, and a 20-step run;
  golden_meta.json   parameters, seeds and scalars of every case, and the
                     SHA-256 of every output field of larger cases
                     (64x32 runs, the rejected-step retry, the moving domain).

Inputs are reproducible without the reference: the init hook's output plus
a numpy default_rng(seed) perturbation, both recorded. Run from the repo
root: python tests/golden/gen_golden.py [reference tree]  (the tree defaults
to FIVONAGI_REF_ROOT, else /root/reference, where this image mounts it).
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from tests.helpers import small_params  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
APPS = {0: "hifu", 1: "taylor", 2: "plane", 3: "focused"}
DTYPES = {"f32": np.float32, "f64": np.float64}


def seeded_input(params, dtype, seed: int, scale: float):
    """Init hook output (from the reference build) plus a seeded perturbation."""
    u = [np.zeros((params.ny, params.nx), dtype) for _ in range(3)]
    oracle.ref_call(params, 0, u, dtype)
    rng = np.random.default_rng(seed)
    return [x + dtype(scale) * rng.standard_normal(x.shape).astype(dtype) for x in u]


def field_hash(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a)
    # -0.0 and +0.0 are the same value; hash values, not sign bits of zeros
    a = np.where(a == 0, np.zeros_like(a), a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def params_dict(p) -> dict:
    return p.as_dict()


def cases_small():
    for app in APPS:
        for key, dt in DTYPES.items():
            yield app, key, dt


def main():
    if not oracle.ref_available():
        tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(oracle.REF_ROOT_ENV, "/root/reference")
        oracle.build_oracle(ref_root=tree)
    arrays = {}
    meta = {"small": [], "hashed": []}
    # ---- 32x16: full grids
    for app, key, dt in cases_small():
        p = small_params(app, 32, 16)
        name = f"{APPS[app]}_{key}"
        u0 = seeded_input(p, dt, seed=app + 1, scale=1e-4)
        init = [np.zeros((p.ny, p.nx), dt) for _ in range(3)]
        oracle.ref_call(p, 0, init, dt)
        for f in range(3):
            arrays[f"{name}_init_u{f + 1}"] = init[f]
            arrays[f"{name}_in_u{f + 1}"] = u0[f]
        for stage in range(4):
            u = [x.copy() for x in u0]
            rc, _ = oracle.ref_call(p, 10 + stage, u, dt)
            assert rc == 0
            for f in range(3):
                arrays[f"{name}_stage{stage}_u{f + 1}"] = u[f]
        u = [x.copy() for x in u0]
        sc = np.array([p.dtini, -p.tide, 0, 0, 0], np.float64)
        rc, st = oracle.ref_call(p, 1, u, dt, nsteps=20, scalars=sc)
        assert rc == 0
        for f in range(3):
            arrays[f"{name}_run20_u{f + 1}"] = u[f]
        meta["small"].append({"name": name, "app": app, "dtype": key, "seed": app + 1, "scale": 1e-4,
                              "params": params_dict(p), "run20": {"dt": sc[0], "T": sc[1], "n": sc[2],
                                                                  "rejected": st["rejected"]}})
    # ---- larger runs, hashed
    larger = [
        ("run60_64x32", lambda app: small_params(app, 64, 32), 60),
        ("run30_32x64", lambda app: small_params(app, 32, 64), 30),
        ("reject_64x32", lambda app: small_params(app, 64, 32).replace(dtini=0.4), 15),
    ]
    for tag, mk, nsteps in larger:
        for app, key, dt in cases_small():
            p = mk(app)
            u = seeded_input(p, dt, seed=10 + app, scale=1e-4)
            sc = np.array([p.dtini, -p.tide, 0, 0, 0], np.float64)
            rc, st = oracle.ref_call(p, 1, u, dt, nsteps=nsteps, scalars=sc)
            assert rc == 0
            meta["hashed"].append({"name": f"{APPS[app]}_{key}_{tag}", "app": app, "dtype": key,
                                   "seed": 10 + app, "scale": 1e-4, "nsteps": nsteps,
                                   "params": params_dict(p), "dt": sc[0], "T": sc[1], "n": sc[2],
                                   "mdx": sc[3], "rejected": st["rejected"],
                                   "sha256": [field_hash(x) for x in u]})
    # moving domain of the taylor-angle-xy app (crosses MDT = 6.25 from T = -4)
    for key, dt in DTYPES.items():
        p = small_params(1, 64, 32).replace(moving_domain=1)
        u = seeded_input(p, dt, seed=99, scale=0.0)
        sc = np.array([p.dtini, -p.tide, 0, 0, 0], np.float64)
        rc, st = oracle.ref_call(p, 1, u, dt, nsteps=90, scalars=sc)
        assert rc == 0 and sc[3] > 0
        meta["hashed"].append({"name": f"taylor_{key}_moving_domain", "app": 1, "dtype": key, "seed": 99,
                               "scale": 0.0, "nsteps": 90, "params": params_dict(p), "dt": sc[0],
                               "T": sc[1], "n": sc[2], "mdx": sc[3], "rejected": st["rejected"],
                               "sha256": [field_hash(x) for x in u]})
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **arrays)
    with open(os.path.join(HERE, "golden_meta.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(f"{len(arrays)} arrays, {len(meta['hashed'])} hashed cases")


if __name__ == "__main__":
    main()
