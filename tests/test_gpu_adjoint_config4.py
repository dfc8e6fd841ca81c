"""The discrete adjoint at config 4 against the oracle's gradients.

Config 4: the phased array on 1024 x 1024 cells, 4000 steps, 128 elements;
loss = mean u1^2 over the 32 x 32 window at (700, 512) over steps
3501-4000; 16 of the 256 weights checked. The fixture
(tests/golden/adjoint_config4.json, made by gen_adjoint_config4.py) holds
the oracle's tangent-linear gradients along the FP32 and FP64 trajectories,
FP64 central differences (h = 1e-4 relative) and the dt schedule.

The GPU adjoint differentiates the FP32 step along the FP32 trajectory, as
the FP32 tangent-linear model does: every checked component within
TLM32_REL of it (measured: 1.3e-4 at most). Against the FP64 gradients --
the tangent-linear model along the FP64 trajectory and the FP64 central
differences, which agree with each other to 2.5e-5 per component -- every
component is within FP64_REL, relative to that component (measured: 8.2e-4
at most; the FP32 tangent-linear model itself sits 6.9e-4 from them). The
GPU's gradient is deterministic (fixed-order reductions), so these bars
are not sampled against noise.
"""
import json
import os

import numpy as np
import pytest

from fivonagi_gb300.adjoint import Adjoint, loss_window

pytestmark = pytest.mark.gpu

TLM32_REL = 1e-3
FP64_REL = 1e-3


def test_config4_gradient_against_the_tangent_linear_model_and_fp64_differences():
    from tests.golden.gen_adjoint_config4 import NSTEPS, SCHED, WINDOW, config4_case, config4_params

    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "adjoint_config4.json")) as f:
        fx = json.load(f)
    p = config4_params()
    amp, ph, dirs = config4_case(p)
    assert list(dirs) == fx["directions"]
    adj = Adjoint(p, loss_window(*WINDOW), NSTEPS)
    loss = adj.forward(amp, ph)
    ga, gp = adj.backward()
    dts, Ts = adj.schedule()
    adj.close()
    sched = np.load(SCHED)
    # the GPU's adaptive schedule is the FP32 oracle's, bit for bit
    assert np.array_equal(dts.astype(np.float32), sched["dts"]) and np.array_equal(Ts.astype(np.float32), sched["Ts"])
    assert abs(loss - fx["loss32"]) <= 1e-9 * fx["loss32"]
    g = np.concatenate([ga, gp])[dirs]
    tlm32 = np.asarray(fx["tlm32"])
    tlm64 = np.asarray(fx["tlm64"])
    fd64 = np.asarray(fx["fd64"])
    rel32 = np.abs(g - tlm32) / np.abs(tlm32)
    rel64 = np.abs(g - tlm64) / np.abs(tlm64)
    relfd = np.abs(g - fd64) / np.abs(fd64)
    print("config 4 gradient, per checked weight: name, GPU adjoint, TLM32, TLM64, FD64, relative distance of the "
          "GPU's to each")
    for r, name in enumerate(fx["direction_names"]):
        print(f"  {name:>12} {g[r]: .8e} {tlm32[r]: .8e} {tlm64[r]: .8e} {fd64[r]: .8e} "
              f"{rel32[r]:.2e} {rel64[r]:.2e} {relfd[r]:.2e}")
    print(f"max rel vs TLM32 {rel32.max():.2e}, vs TLM64 {rel64.max():.2e}, vs FD64 {relfd.max():.2e}")
    assert np.all(rel32 <= TLM32_REL), rel32
    assert np.all(rel64 <= FP64_REL), rel64
    assert np.all(relfd <= FP64_REL), relfd
