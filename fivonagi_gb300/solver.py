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

    def set_array_weights(self, amp, phase) -> None:
        """Phased-array element amplitudes and phases (FP32)."""
        a = np.ascontiguousarray(amp, np.float32)
        ph = np.ascontiguousarray(phase, np.float32)
        fp = C.POINTER(C.c_float)
        check(self.lib.fv_set_array_weights(self.h, a.ctypes.data_as(fp), ph.ctypes.data_as(fp), int(a.size)),
              "fv_set_array_weights")

    def filter_u1(self, radius: float) -> np.ndarray:
        """The current u1 low-pass filtered in Fourier space (fv_filter_u1)."""
        out = np.empty(self.shape, np.float32)
        check(self.lib.fv_filter_u1(self.h, float(radius), out.ctypes.data, 0), "fv_filter_u1")
        return out

    def render(self, width=None, height=None, zoom: int = 1, i0: int = 0, j0: int = 0, jcut: int = -1,
               overlays: bool = False, plot_scale: float = 1.0) -> np.ndarray:
        """The headless display (fv_render): an RGBA8 image, rows first."""
        spec = _abi.FvRenderSpec()
        spec.width = int(width or self.params.nx // zoom)
        spec.height = int(height or self.params.ny // zoom)
        spec.zoom, spec.i0, spec.j0, spec.jcut = int(zoom), int(i0), int(j0), int(jcut)
        spec.overlays, spec.plot_scale = int(bool(overlays)), float(plot_scale)
        rows = spec.height + (128 if jcut >= 0 else 0)
        out = np.zeros((rows, spec.width, 4), np.uint8)
        check(self.lib.fv_render(self.h, C.byref(spec), out.ctypes.data, 0), "fv_render")
        return out

    def collect_enable(self, probes=(), envelope_row: int = -1, envelope_len: int = 0, capacity: int = 0,
                       envelope_halfwidth: float = 0.0) -> None:
        """On-device collection after each accepted step (fv_collect_enable):
        probes = [(i_lab, j_lab), ...] (at most 8); the u1 envelope along lab
        row envelope_row; capacity steps between reads (default NX)."""
        spec = _abi.FvCollectSpec()
        spec.nprobes = len(probes)
        for k, (i, j) in enumerate(probes):
            spec.probe_i[k], spec.probe_j[k] = int(i), int(j)
        spec.envelope_row = int(envelope_row)
        spec.envelope_len = int(envelope_len or self.params.nx)
        spec.capacity = int(capacity or self.params.nx)
        spec.envelope_halfwidth = float(envelope_halfwidth)
        self._collect = spec
        check(self.lib.fv_collect_enable(self.h, C.byref(spec)), "fv_collect_enable")

    def collect_disable(self) -> None:
        check(self.lib.fv_collect_enable(self.h, None), "fv_collect_enable")
        self._collect = None

    def collect_read(self) -> dict:
        """The series since the last read (T, cfl, probes [steps, nprobes])
        and the envelope; empties the series."""
        spec = self._collect
        cap = spec.capacity
        T = np.zeros(cap, np.float32)
        cfl = np.zeros(cap, np.float32)
        probes = np.zeros((cap, 8), np.float32)
        env = np.zeros(max(spec.envelope_len, 1), np.float32)
        n = C.c_int32()
        fp = C.POINTER(C.c_float)
        check(self.lib.fv_collect_read(self.h, C.byref(n), T.ctypes.data_as(fp), cfl.ctypes.data_as(fp),
                                       probes.ctypes.data_as(fp), env.ctypes.data_as(fp)), "fv_collect_read")
        k = n.value
        return {"steps": k, "T": T[:k], "cfl": cfl[:k], "probes": probes[:k, :spec.nprobes],
                "envelope": env[:spec.envelope_len] if spec.envelope_row >= 0 else None}

    def snapshot(self) -> None:
        """Save the state and time-stepping scalars (one slot)."""
        check(self.lib.fv_snapshot(self.h), "fv_snapshot")

    def restore(self) -> None:
        """Return to the last snapshot."""
        check(self.lib.fv_restore(self.h), "fv_restore")

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

    def time_attempts(self, n: int) -> tuple[float, float]:
        """(step kernel ms, attempt ms), averaged over n attempts launched
        one at a time with CUDA events between their launches
        (fv_time_attempts)."""
        sk, at = C.c_float(), C.c_float()
        check(self.lib.fv_time_attempts(self.h, int(n), C.byref(sk), C.byref(at)), "fv_time_attempts")
        return sk.value, at.value

    def time_run(self, n: int) -> float:
        """Device ms of n attempts launched as launch_attempts does (CUDA
        events on the handle's stream; fv_time_run). Synchronises."""
        ms = C.c_float()
        check(self.lib.fv_time_run(self.h, int(n), C.byref(ms)), "fv_time_run")
        return ms.value

    def sync(self) -> dict:
        st = FvRunStats()
        check(self.lib.fv_sync(self.h, C.byref(st)), "fv_sync")
        return st.as_dict()

    def steps_async(self, n: int) -> None:
        """Enqueue n attempts without synchronising (fv_steps_async; at most
        64 in flight)."""
        check(self.lib.fv_steps_async(self.h, int(n)), "fv_steps_async")

    def step_wait(self) -> dict:
        """Stats of the oldest attempt in flight, once it has completed
        (fv_step_wait)."""
        st = FvRunStats()
        check(self.lib.fv_step_wait(self.h, C.byref(st)), "fv_step_wait")
        return st.as_dict()

    def steps_pipelined(self, n: int, block: int = 32):
        """n attempts with every attempt's stats read back, the next block of
        attempts enqueued before the current block is read; yields each
        attempt's stats in order."""
        block = max(1, min(block, 32))
        queued = min(n, block)
        if queued:
            self.steps_async(queued)
        for k in range(n):
            if k % block == 0 and queued < n:
                m = min(block, n - queued)
                self.steps_async(m)
                queued += m
            yield self.step_wait()

    def set_launch(self, blocks: int) -> None:
        """CTAs per step launch (0 = default); see fv_set_launch."""
        check(self.lib.fv_set_launch(self.h, int(blocks)), "fv_set_launch")

    def get_launch(self) -> tuple[int, int]:
        """(CTAs per launch, CTAs resident at once on this device)."""
        b, m = C.c_int32(), C.c_int32()
        check(self.lib.fv_get_launch(self.h, C.byref(b), C.byref(m)), "fv_get_launch")
        return b.value, m.value

    def set_cta_shape(self, shape: int) -> None:
        """The step kernel's CTA shape (fv_set_cta_shape); resets the CTA
        count to the shape's default."""
        check(self.lib.fv_set_cta_shape(self.h, int(shape)), "fv_set_cta_shape")

    def get_cta_shape(self) -> tuple[int, int]:
        """(shape, warps per CTA) of the step kernel."""
        s, w = C.c_int32(), C.c_int32()
        check(self.lib.fv_get_cta_shape(self.h, C.byref(s), C.byref(w)), "fv_get_cta_shape")
        return s.value, w.value

    def set_division(self, mode: int) -> None:
        """Division in the step kernel (fv_set_division): _abi.FV_DIVISION_FMA,
        FV_DIVISION_EXACT or FV_DIVISION_DEFAULT; results are the same."""
        check(self.lib.fv_set_division(self.h, int(mode)), "fv_set_division")

    def get_division(self) -> int:
        m = C.c_int32()
        check(self.lib.fv_get_division(self.h, C.byref(m)), "fv_get_division")
        return m.value

    def debug_step(self, stage: int):
        """One step of the current state stopped after `stage` (no commit)."""
        out = [np.empty(self.shape, np.float32) for _ in range(3)]
        check(self.lib.fv_debug_step(self.h, int(stage), *[a.ctypes.data for a in out]), "fv_debug_step")
        return out


class Batch:
    """n independent simulations stepped together (fv_batch_*)."""

    def __init__(self, params_list):
        self.lib = _abi.load_library()
        self.params = [p.copy() for p in params_list]
        self.n = len(self.params)
        arr = (FvParams * self.n)(*self.params)
        h = C.c_void_p()
        check(self.lib.fv_batch_create(self.n, arr, C.byref(h)), "fv_batch_create")
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.fv_batch_destroy(self.h)
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

    def shape(self, k: int):
        return (self.params[k].ny, self.params[k].nx)

    def init_state(self) -> None:
        check(self.lib.fv_batch_init_state(self.h), "fv_batch_init_state")

    def set_state(self, k: int, u1, u2, u3) -> None:
        arrs = [np.ascontiguousarray(u, dtype=np.float32).reshape(self.shape(k)) for u in (u1, u2, u3)]
        check(self.lib.fv_batch_set_state(self.h, k, *[a.ctypes.data for a in arrs], 0), "fv_batch_set_state")

    def get_state(self, k: int):
        out = [np.empty(self.shape(k), np.float32) for _ in range(3)]
        check(self.lib.fv_batch_get_state(self.h, k, *[a.ctypes.data for a in out], 0), "fv_batch_get_state")
        return out

    def set_stream(self, stream_ptr: int | None) -> None:
        check(self.lib.fv_batch_set_stream(self.h, stream_ptr), "fv_batch_set_stream")

    def run(self, nsteps: int) -> list[dict]:
        st = (FvRunStats * self.n)()
        check(self.lib.fv_batch_run(self.h, int(nsteps), st), "fv_batch_run")
        return [s.as_dict() for s in st]

    def run_status(self, nsteps: int) -> tuple[int, list[dict]]:
        """Like run, but returns (status, stats) instead of raising."""
        st = (FvRunStats * self.n)()
        rc = self.lib.fv_batch_run(self.h, int(nsteps), st)
        return rc, [s.as_dict() for s in st]

    def launch_attempts(self, n: int) -> None:
        check(self.lib.fv_batch_launch_attempts(self.h, int(n)), "fv_batch_launch_attempts")

    def time_run(self, n: int) -> float:
        """Device ms of n attempts of every simulation, launched as
        launch_attempts does (fv_batch_time_run). Synchronises."""
        ms = C.c_float()
        check(self.lib.fv_batch_time_run(self.h, int(n), C.byref(ms)), "fv_batch_time_run")
        return ms.value

    def sync(self) -> list[dict]:
        st = (FvRunStats * self.n)()
        check(self.lib.fv_batch_sync(self.h, st), "fv_batch_sync")
        return [s.as_dict() for s in st]

    def set_launch(self, blocks: int) -> None:
        check(self.lib.fv_batch_set_launch(self.h, int(blocks)), "fv_batch_set_launch")

    def get_launch(self) -> tuple[int, int]:
        b, m = C.c_int32(), C.c_int32()
        check(self.lib.fv_batch_get_launch(self.h, C.byref(b), C.byref(m)), "fv_batch_get_launch")
        return b.value, m.value
