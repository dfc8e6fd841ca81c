"""Gradients of a windowed pressure loss with respect to the phased array's
element weights, through the C ABI's discrete adjoint (fv_adjoint_*).

`Adjoint` owns one fv_adjoint: forward(amp, phase) -> loss runs the
recorded forward; backward() -> (d loss/d amp, d loss/d phase) runs the
reverse pass; replay(amp, phase) -> loss re-runs the forward on the
recorded dt schedule (finite differences). `ArrayLoss` exposes the same to
torch.autograd; it does no arithmetic of its own. `AdjointBatch` owns one
fv_adjoint_batch: many designs of one grid in one launch sequence.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import FvLossWindow, FvParams, check


def loss_window(i0: int, j0: int, ni: int, nj: int, step_first: int, step_last: int) -> FvLossWindow:
    w = FvLossWindow()
    w.i0, w.j0, w.ni, w.nj = int(i0), int(j0), int(ni), int(nj)
    w.step_first, w.step_last = int(step_first), int(step_last)
    return w


def _f32(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


class Adjoint:
    def __init__(self, params: FvParams, window: FvLossWindow, nsteps: int, checkpoint_every: int = 0):
        self.lib = _abi.load_library()
        self.params = params.copy()
        self.window = window
        self.nsteps = int(nsteps)
        self.nelem = int(params.array_elems)
        self.h = C.c_void_p()
        p = self.params
        check(self.lib.fv_adjoint_create(C.byref(p), C.byref(window), self.nsteps, int(checkpoint_every),
                                         C.byref(self.h)), "fv_adjoint_create")

    def close(self) -> None:
        if self.h:
            self.lib.fv_adjoint_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, cuda_stream: int) -> None:
        check(self.lib.fv_adjoint_set_stream(self.h, C.c_void_p(cuda_stream)), "fv_adjoint_set_stream")

    def forward(self, amp, phase) -> float:
        a, pa = _f32(amp)
        ph, pph = _f32(phase)
        loss = C.c_double()
        check(self.lib.fv_adjoint_forward(self.h, pa, pph, C.byref(loss)), "fv_adjoint_forward")
        return loss.value

    def replay(self, amp, phase) -> float:
        a, pa = _f32(amp)
        ph, pph = _f32(phase)
        loss = C.c_double()
        check(self.lib.fv_adjoint_replay(self.h, pa, pph, C.byref(loss)), "fv_adjoint_replay")
        return loss.value

    def backward(self):
        ga = np.zeros(self.nelem, np.float64)
        gp = np.zeros(self.nelem, np.float64)
        dp = C.POINTER(C.c_double)
        check(self.lib.fv_adjoint_backward(self.h, ga.ctypes.data_as(dp), gp.ctypes.data_as(dp)),
              "fv_adjoint_backward")
        return ga, gp

    def schedule(self):
        dt = np.zeros(self.nsteps, np.float64)
        T = np.zeros(self.nsteps, np.float64)
        dp = C.POINTER(C.c_double)
        check(self.lib.fv_adjoint_schedule(self.h, dt.ctypes.data_as(dp), T.ctypes.data_as(dp)),
              "fv_adjoint_schedule")
        return dt, T

    def get_state(self):
        shape = (self.params.ny, self.params.nx)
        out = [np.empty(shape, np.float32) for _ in range(3)]
        fp = C.POINTER(C.c_float)
        check(self.lib.fv_adjoint_get_state(self.h, *[o.ctypes.data_as(fp) for o in out]), "fv_adjoint_get_state")
        return out


class AdjointBatch:
    """D designs of one grid through one fv_adjoint_batch: forward(amp,
    phase) with (D, nelem) arrays -> D losses; backward() -> (D, nelem)
    gradients of amplitudes and phases. Each design's results equal the
    single-design Adjoint's for it, bit for bit."""

    def __init__(self, params: FvParams, windows, nsteps: int, checkpoint_every: int = 0):
        self.lib = _abi.load_library()
        self.params = params.copy()
        self.nd = len(windows)
        self.nsteps = int(nsteps)
        self.nelem = int(params.array_elems)
        self.windows = (FvLossWindow * self.nd)(*windows)
        self.h = C.c_void_p()
        p = self.params
        check(self.lib.fv_adjoint_batch_create(C.byref(p), self.nd, self.windows, self.nsteps, int(checkpoint_every),
                                               C.byref(self.h)), "fv_adjoint_batch_create")

    def close(self) -> None:
        if self.h:
            self.lib.fv_adjoint_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, cuda_stream: int) -> None:
        check(self.lib.fv_adjoint_batch_set_stream(self.h, C.c_void_p(cuda_stream)), "fv_adjoint_batch_set_stream")

    def forward(self, amp, phase) -> np.ndarray:
        a, pa = _f32(np.asarray(amp).reshape(self.nd, self.nelem))
        ph, pph = _f32(np.asarray(phase).reshape(self.nd, self.nelem))
        loss = np.zeros(self.nd, np.float64)
        check(self.lib.fv_adjoint_batch_forward(self.h, pa, pph, loss.ctypes.data_as(C.POINTER(C.c_double))),
              "fv_adjoint_batch_forward")
        return loss

    def backward(self):
        ga = np.zeros((self.nd, self.nelem), np.float64)
        gp = np.zeros((self.nd, self.nelem), np.float64)
        dp = C.POINTER(C.c_double)
        check(self.lib.fv_adjoint_batch_backward(self.h, ga.ctypes.data_as(dp), gp.ctypes.data_as(dp)),
              "fv_adjoint_batch_backward")
        return ga, gp

    def schedule(self, design: int):
        dt = np.zeros(self.nsteps, np.float64)
        T = np.zeros(self.nsteps, np.float64)
        dp = C.POINTER(C.c_double)
        check(self.lib.fv_adjoint_batch_schedule(self.h, int(design), dt.ctypes.data_as(dp), T.ctypes.data_as(dp)),
              "fv_adjoint_batch_schedule")
        return dt, T


def array_loss_function():
    """torch.autograd.Function over an Adjoint: loss = f(amp, phase)."""
    import torch

    class ArrayLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, amp, phase, adj: Adjoint):
            loss = adj.forward(amp.detach().cpu().numpy(), phase.detach().cpu().numpy())
            ctx.adj = adj
            ctx.device, ctx.dtype = amp.device, amp.dtype
            return torch.tensor(loss, dtype=torch.float64, device=amp.device)

        @staticmethod
        def backward(ctx, grad_out):
            ga, gp = ctx.adj.backward()
            g = grad_out.detach().to("cpu", torch.float64)
            to = dict(device=ctx.device, dtype=ctx.dtype)
            return (torch.as_tensor(ga, dtype=torch.float64).mul(g).to(**to),
                    torch.as_tensor(gp, dtype=torch.float64).mul(g).to(**to), None)

    return ArrayLoss
