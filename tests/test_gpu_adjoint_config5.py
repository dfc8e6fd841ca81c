"""The batched adjoint at config 5 against the FP64 oracle, for one design.

Config 5: designs of the phased array on 2048 x 1024 cells, 6000 steps,
128 elements, each design with its own weights and focal window (as
bench.py's designs workload builds them). Design 0 runs here inside a
batch of two designs, so the gradient checked is the batched adjoint's.
The fixture (tests/golden/adjoint_config5.json, made by
gen_adjoint_config5.py) holds FP64 central differences (h = 1e-4
relative) of design 0's loss on its dt schedule, for 4 of its 256
weights, and the schedule itself: the batch must reproduce the schedule bit
for bit and the FP32 loss, and each checked gradient component must lie
within FP64_REL of the FP64 one, relative to that component (measured:
5.4e-4 at most; the FP32 trajectory's own error sets the distance, up to
8e-4 at config 4). The batched gradient is deterministic.
"""
import json
import os

import numpy as np
import pytest

from fivonagi_gb300.adjoint import AdjointBatch, loss_window

pytestmark = pytest.mark.gpu

FP64_REL = 1e-3


def test_config5_design_gradient_against_fp64_differences():
    from tests.golden.gen_adjoint_config5 import NSTEPS, SCHED, config5_case, config5_params

    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "adjoint_config5.json")) as f:
        fx = json.load(f)
    p = config5_params()
    cases = [config5_case(p, d) for d in (0, 1)]
    assert list(cases[0][3]) == fx["directions"]
    amp = np.stack([c[0] for c in cases])
    ph = np.stack([c[1] for c in cases])
    ab = AdjointBatch(p, [loss_window(*c[2]) for c in cases], NSTEPS)
    loss = ab.forward(amp, ph)
    ga, gp = ab.backward()
    dts, Ts = ab.schedule(0)
    ab.close()
    sched = np.load(SCHED)
    assert np.array_equal(dts.astype(np.float32), sched["dts"]) and np.array_equal(Ts.astype(np.float32), sched["Ts"])
    assert abs(loss[0] - fx["loss32"]) <= 1e-9 * fx["loss32"]
    g = np.concatenate([ga[0], gp[0]])[np.asarray(fx["directions"])]
    fd64 = np.asarray(fx["fd64"])
    rel = np.abs(g - fd64) / np.abs(fd64)
    print("config 5, design 0 in a batch of 2: name, batched adjoint, FD64, relative distance")
    for r, name in enumerate(fx["direction_names"]):
        print(f"  {name:>12} {g[r]: .8e} {fd64[r]: .8e} {rel[r]:.2e}")
    print(f"max rel vs FD64 {rel.max():.2e}")
    assert np.all(rel <= FP64_REL), rel
