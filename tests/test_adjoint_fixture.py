"""The config-4 gradient fixture pinned against itself, on CPU.

tests/golden/adjoint_config4.json holds, for 16 of the phased array's 256
weights at config 4 (1024 x 1024, 4000 steps), the oracle's tangent-linear
gradient along the FP32 and the FP64 trajectories and FP64 central
differences (h = 1e-4 relative) of the loss on the same frozen dt schedule
(gen_adjoint_config4.py). The FP64 tangent-linear model and the central
differences are independent routes to the same derivative: their per-
component agreement pins the oracle's tangent-linear model (the dual-number
restatement of the step), which the GPU adjoint is then held to
(test_gpu_adjoint_config4.py).
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture():
    with open(os.path.join(HERE, "golden", "adjoint_config4.json")) as f:
        return json.load(f)


def test_fp64_tangent_linear_model_agrees_with_fp64_central_differences():
    fx = _fixture()
    tlm64, fd64 = np.asarray(fx["tlm64"]), np.asarray(fx["fd64"])
    assert len(tlm64) == len(fd64) == 16 and np.all(np.isfinite(fd64))
    rel = np.abs(tlm64 - fd64) / np.abs(fd64)
    assert rel.max() <= 1e-4, rel  # measured 2.5e-5: the O(h^2) error of the differences


def test_fp32_and_fp64_gradients_differ_by_the_fp32_trajectory_error():
    """Along the FP32 trajectory the gradient moves by about the FP32 state
    error (~1e-4 relative): well below the adjoint's 1e-3 bar, well above
    rounding of the derivative arithmetic itself (done in double)."""
    fx = _fixture()
    tlm32, tlm64 = np.asarray(fx["tlm32"]), np.asarray(fx["tlm64"])
    rel = np.abs(tlm32 - tlm64) / np.abs(tlm64)
    assert 1e-7 < rel.max() <= 1e-3, rel
    assert abs(fx["loss32"] - fx["loss64"]) <= 1e-3 * fx["loss64"]


def test_directions_and_steps():
    fx = _fixture()
    case = fx["case"]
    assert (case["nx"], case["ny"], case["nsteps"], case["elements"]) == (1024, 1024, 4000, 128)
    assert len(set(fx["directions"])) == 16 and all(0 <= k < 256 for k in fx["directions"])
    h = np.asarray(fx["fd64_h"])
    assert np.all(h > 0)


def test_fixture_parameters_are_the_library_defaults():
    """The generators build the phased array's parameters without the
    library (the oracle runs on the host); they must be the library's own
    defaults, with config 5's grid as bench.py's designs workload sets it."""
    from fivonagi_gb300 import _abi
    from tests.golden.gen_adjoint_config4 import config4_params
    from tests.golden.gen_adjoint_config5 import config5_params

    lib = _abi.default_params("phased-array")
    assert config4_params().as_dict() == lib.as_dict()
    c5 = lib.replace(nx=2048, ny=1024, xmax=2047 / 24, ymax=1023 / 24, center=512.0)
    assert config5_params().as_dict() == c5.as_dict()


def test_config5_fixture_is_complete():
    with open(os.path.join(HERE, "golden", "adjoint_config5.json")) as f:
        fx = json.load(f)
    case = fx["case"]
    assert (case["nx"], case["ny"], case["nsteps"], case["design"]) == (2048, 1024, 6000, 0)
    fd = np.asarray(fx["fd64"])
    assert len(fd) == len(fx["directions"]) == 4 and np.all(np.isfinite(fd)) and np.all(fd != 0)
    assert fx["loss32"] > 0
    z = np.load(os.path.join(HERE, "golden", "adjoint_config5_schedule.npz"))
    assert z["dts"].shape == z["Ts"].shape == (6000,) and np.all(z["dts"] > 0) and np.all(np.diff(z["Ts"]) > 0)
