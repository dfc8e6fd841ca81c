"""fv_step_noalloc: a step attempt that allocates no device memory.

Some callers cannot let the library call cudaMalloc -- programs whose device
memory belongs to their own allocator (a framework's caching allocator or a
fixed arena). For them fv_step_noalloc takes caller-owned input and output
buffers and keeps the step kernel's scratch in a fixed __device__ array.
This test calls it through the C ABI on device buffers the test owns and
checks its output, dt, T and window offsets against the allocating path
(fv_create + fv_run), bit for bit, on calls in a row (each reuses the
scratch array the previous one left behind): two plain steps of three apps
in both arithmetic variants, steps past the moving window's start, and
rejected attempts retried with the returned dt.

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


def _device_state(u0):
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    src = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in u0]
    dst = [torch.full_like(x, float("nan")) for x in src]
    torch.cuda.synchronize()
    return src, dst


def _chain(lib, p, u0, calls):
    """`calls` accepted steps through fv_step_noalloc, each retried with
    res.dt_next after a rejection (the caller bounds its retries), compared
    after every accepted step with fv_run(1) of an fv_create handle."""
    sim = Simulation(p)
    sim.set_state(*u0)
    src, dst = _device_state(u0)
    res = _abi.FvStepResult()
    dt, T, mdx, mdy = p.dtini, -p.tide, 0, 0
    rejected = 0
    total_rejected = 0  # fv_run's own retries (each run's stats count that run's attempts)
    for call in range(calls):
        for _retry in range(8):
            rc = lib.fv_step_noalloc(C.byref(p), *[x.data_ptr() for x in src], *[x.data_ptr() for x in dst],
                                     dt, T, mdx, mdy, None, C.byref(res))
            assert rc == _abi.FV_OK, lib.fv_last_error_string()
            assert res.status == 0
            if res.accepted:
                break
            # a rejected attempt leaves T and the window alone and gives
            # update_dt's retry step
            rejected += 1
            assert np.float32(res.T) == np.float32(T) and (res.mdx, res.mdy) == (mdx, mdy)
            assert res.dt_next <= float(np.float32(dt)) * 0.9 * (1 + 1e-6)
            dt = res.dt_next
        assert res.accepted == 1
        st = sim.run(1)
        total_rejected += st["rejected"]
        ref = sim.get_state()
        for f in range(3):
            got = dst[f].cpu().numpy()
            assert same_values(got, ref[f]), f"call {call} field {f}: rel L2 {rel_l2(got, ref[f]):.3e}"
        assert np.float32(res.dt_next) == np.float32(st["dt"])
        assert np.float32(res.T) == np.float32(st["T"])
        assert np.float32(res.cfl) == np.float32(st["cfl"])
        assert (res.mdx, res.mdy) == (st["mdx"], st["mdy"])
        src, dst = dst, src
        dt, T, mdx, mdy = res.dt_next, res.T, res.mdx, res.mdy
    sim.close()
    return rejected, total_rejected, mdx


@pytest.mark.parametrize("app,nx,ny,exact", [(3, 300, 130, 1), (2, 64, 32, 1), (0, 100, 37, 1), (3, 300, 130, 0)])
def test_noalloc_matches_fv_run_on_two_calls(app, nx, ny, exact):
    lib = _abi.load_library()
    p = small_params(app, nx, ny, exact=exact)
    orc = OracleSim(p, np.float32, math="fvm")
    orc.init_state()
    u0 = perturbed(orc.get_state(), 9, 1e-4)
    _chain(lib, p, u0, 2)


def test_noalloc_moving_window_shift_matches_fv_run():
    """Steps past MDT: the window shifts inside the step, as with fv_run."""
    lib = _abi.load_library()
    p = small_params(2, 64, 32).replace(moving_domain=1, mdt=0.05, mdvx=1.0, mdvy=0.25)
    orc = OracleSim(p, np.float32, math="fvm")
    orc.init_state()
    u0 = perturbed(orc.get_state(), 4, 1e-4)
    _, _, mdx = _chain(lib, p, u0, 40)
    assert mdx > 0


def test_noalloc_rejected_attempt_is_retried_like_fv_run():
    """A first dt far above the CFL limit: rejected attempts return
    accepted = 0 and the retry dt; the accepted step then equals fv_run's,
    which retried inside the library the same number of times."""
    lib = _abi.load_library()
    p = small_params(2, 64, 32).replace(dtini=0.3)
    orc = OracleSim(p, np.float32, math="fvm")
    orc.init_state()
    rejected, total, _ = _chain(lib, p, orc.get_state(), 3)
    assert rejected >= 1 and rejected == total


def test_noalloc_rejects_aliased_buffers():
    import torch

    lib = _abi.load_library()
    p = small_params(2, 64, 32)
    res = _abi.FvStepResult()
    bufs = [torch.zeros(p.nx * p.ny, device="cuda") for _ in range(3)]
    ptrs = [b.data_ptr() for b in bufs]
    # the host rejects the aliasing before any device work
    rc = lib.fv_step_noalloc(C.byref(p), *ptrs, *ptrs, 0.01, 0.0, 0, 0, None, C.byref(res))
    assert rc == _abi.FV_BAD_ARG
    assert b"also an input" in lib.fv_last_error_string()


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
