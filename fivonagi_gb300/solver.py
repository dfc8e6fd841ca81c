"""Python host mirror of the reference's per-app driver, over the C ABI.

The reference's driver is common/main.cu: main() sets dt = DTINI,
T = -TIDE, runs the app's init() on the host and uploads the state
(:789-876), then calls calcFrame() forever, each call advancing until
T >= Tprint and Tprint += DTPRINT (:247-756). `Simulation` offers the same
sequence -- init_state(), calc_frame() -- plus run(nsteps) and per-stage
debug steps, all through libfivonagi.so. No arithmetic happens here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import FvParams, FvRunStats, check


class Simulation:
    """One simulation on the current CUDA device (one fv_handle)."""

    def __init__(self, params: FvParams | None = None, app: int | str | None = None, **overrides):
        self.lib = _abi.load_library()
        if params is None:
            if app is None:
                raise ValueError("give params or app")
            params = _abi.default_params(app)
        params = params.replace(**overrides) if overrides else params.copy()
        self.params = params
        self.shape = (params.ny, params.nx)
        h = C.c_void_p()
        check(self.lib.fv_create(C.byref(self.params), C.byref(h)), "fv_create")
        self.h = h
        self.tprint = None

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.fv_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state
    def init_state(self) -> None:
        """The app's init hook; dt = DTINI, T = -TIDE, n = 0."""
        check(self.lib.fv_init_state(self.h), "fv_init_state")
        self.tprint = None

    def set_state(self, u1, u2, u3) -> None:
        arrs = [np.ascontiguousarray(u, dtype=np.float32).reshape(self.shape) for u in (u1, u2, u3)]
        check(self.lib.fv_set_state(self.h, *[a.ctypes.data for a in arrs], 0), "fv_set_state")
        self.tprint = None

    def set_state_device(self, p1: int, p2: int, p3: int) -> None:
        """Device pointers (e.g. torch tensor .data_ptr()) of NX*NY floats each."""
        check(self.lib.fv_set_state(self.h, p1, p2, p3, 1), "fv_set_state")
        self.tprint = None

    def get_state(self):
        out = [np.empty(self.shape, np.float32) for _ in range(3)]
        check(self.lib.fv_get_state(self.h, *[a.ctypes.data for a in out], 0), "fv_get_state")
        return out

    def get_state_device(self, p1: int, p2: int, p3: int) -> None:
        check(self.lib.fv_get_state(self.h, p1, p2, p3, 1), "fv_get_state")

    def set_scalars(self, dt: float, T: float, n: int = 0) -> None:
        check(self.lib.fv_set_scalars(self.h, float(dt), float(T), int(n)), "fv_set_scalars")

    def stats(self) -> dict:
        st = FvRunStats()
        check(self.lib.fv_get_stats(self.h, C.byref(st)), "fv_get_stats")
        return st.as_dict()

    def set_stream(self, stream_ptr: int | None) -> None:
        check(self.lib.fv_set_stream(self.h, stream_ptr), "fv_set_stream")

    # -- time stepping
    def run(self, nsteps: int) -> dict:
        """Exactly nsteps accepted steps (rejected attempts are retried)."""
        st = FvRunStats()
        check(self.lib.fv_run(self.h, int(nsteps), C.byref(st)), "fv_run")
        return st.as_dict()

    def run_until(self, t_stop: float) -> dict:
        st = FvRunStats()
        check(self.lib.fv_run_until(self.h, float(t_stop), C.byref(st)), "fv_run_until")
        return st.as_dict()

    def calc_frame(self, dtprint: float = 1.0) -> dict:
        """Advance until T >= Tprint, then Tprint += DTPRINT (calcFrame)."""
        if self.tprint is None:
            self.tprint = self.stats()["T"] + dtprint
        st = self.run_until(self.tprint)
        self.tprint += dtprint
        return st

    def launch_attempts(self, n: int) -> None:
        check(self.lib.fv_launch_attempts(self.h, int(n)), "fv_launch_attempts")

    def sync(self) -> dict:
        st = FvRunStats()
        check(self.lib.fv_sync(self.h, C.byref(st)), "fv_sync")
        return st.as_dict()

    def debug_step(self, stage: int):
        """One step of the current state stopped after `stage` (no commit)."""
        out = [np.empty(self.shape, np.float32) for _ in range(3)]
        check(self.lib.fv_debug_step(self.h, int(stage), *[a.ctypes.data for a in out]), "fv_debug_step")
        return out
