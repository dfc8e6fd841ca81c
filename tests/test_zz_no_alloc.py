"""fv_step_noalloc: a step attempt that allocates no device memory.

Some callers cannot let the library call cudaMalloc -- programs whose device
memory belongs to their own allocator (a framework's caching allocator or a
fixed arena). For them fv_step_noalloc takes caller-owned input and output
buffers and keeps the step kernel's scratch in a fixed __device__ array.
This test calls it through the C ABI on device buffers the test owns and
checks its output, dt and T against the allocating path (fv_create +
fv_run), bit for bit, on two calls in a row; the second call reuses the
scratch array the first one left behind.

The file is named to be collected last, so that a run stopping at the first
failure has already run every other test; it also passes alone in a fresh
process (the first call does the per-device set-up).
"""
import ctypes as C

import numpy as np
import pytest

from fivonagi_gb300 import Simulation, _abi
from oracle.oracle import OracleSim
from tests.helpers import perturbed, rel_l2, same_values, small_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("app,nx,ny", [(3, 300, 130), (2, 64, 32), (0, 100, 37)])
def test_noalloc_matches_fv_run_on_two_calls(app, nx, ny):
    import torch

    lib = _abi.load_library()
    p = small_params(app, nx, ny)
    orc = OracleSim(p, np.float32, math="fvm")
    orc.init_state()
    u0 = perturbed(orc.get_state(), 9, 1e-4)
    sim = Simulation(p)
    sim.set_state(*u0)
    dev = torch.device("cuda", torch.cuda.current_device())
    src = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in u0]
    dst = [torch.full_like(x, float("nan")) for x in src]
    torch.cuda.synchronize()
    res = _abi.FvStepResult()
    dt, T, mdx, mdy = p.dtini, -p.tide, 0, 0
    for call in range(2):
        rc = lib.fv_step_noalloc(C.byref(p), *[x.data_ptr() for x in src], *[x.data_ptr() for x in dst],
                                 dt, T, mdx, mdy, None, C.byref(res))
        assert rc == _abi.FV_OK, lib.fv_last_error_string()
        assert res.accepted == 1 and res.status == 0
        st = sim.run(1)
        ref = sim.get_state()
        for f in range(3):
            got = dst[f].cpu().numpy()
            assert same_values(got, ref[f]), f"call {call} field {f}: rel L2 {rel_l2(got, ref[f]):.3e}"
        assert np.float32(res.dt_next) == np.float32(st["dt"])
        assert np.float32(res.T) == np.float32(st["T"])
        assert np.float32(res.cfl) == np.float32(st["cfl"])
        src, dst = dst, src
        dt, T, mdx, mdy = res.dt_next, res.T, res.mdx, res.mdy
    sim.close()


def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch

    lib = _abi.load_library()
    p = small_params(2, 64, 32).replace(nx=12000, ny=8000)  # nx + ny > FV_NOALLOC_MAX_PERIMETER
    res = _abi.FvStepResult()
    # the host rejects the size before any device work; the buffers are never touched
    bufs = [torch.zeros(8, device="cuda") for _ in range(6)]
    rc = lib.fv_step_noalloc(C.byref(p), *[b.data_ptr() for b in bufs], 0.01, 0.0, 0, 0, None, C.byref(res))
    assert rc == _abi.FV_BAD_ARG
    assert b"FV_NOALLOC_MAX_PERIMETER" in lib.fv_last_error_string()
