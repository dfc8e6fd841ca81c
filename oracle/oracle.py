"""ctypes loader for the oracle libraries. TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this module, as the checker and the CPU baseline; the product package
(fivonagi_gb300) never imports it.

  OracleSim  -- the CPU restatement (oracle/fv_oracle.cpp, built into
                oracle/_build/liboracle.so), FP32 or FP64.
  ref_run    -- the reference's own headers built on the host through
                oracle/ref_shim.cpp (oracle/_ref/libfvref.so); exists only
                where the reference tree was present at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from fivonagi_gb300._abi import FvParams, FvRunStats

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libfvref.so")
# where the reference source tree is, for the host build of its headers
REF_ROOT_ENV = "FIVONAGI_REF_ROOT"

REF_APP_KEYS = {0: "hifu", 1: "taylor", 2: "plane", 3: "focused"}

_oracle = None
_ref = None


def build_oracle(ref_root: str | None = None, with_ref: bool = True) -> None:
    """Compile the restatement, and the reference shim when a reference tree
    is given (`ref_root`, or the FIVONAGI_REF_ROOT environment variable) and
    exists."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    root = ref_root or os.environ.get(REF_ROOT_ENV)
    if with_ref and root and os.path.isdir(os.path.join(root, "apps", "na")):
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF_ROOT={root}"], check=True)


def _load_oracle() -> C.CDLL:
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB):
            build_oracle(with_ref=False)
        lib = C.CDLL(ORACLE_LIB)
        P = C.c_void_p
        lib.fvo_create.restype = P
        lib.fvo_create.argtypes = [C.POINTER(FvParams), C.c_int, C.c_int]
        lib.fvo_destroy.argtypes = [P]
        lib.fvo_set_threads.restype = C.c_int
        lib.fvo_set_threads.argtypes = [C.c_int]
        for name in ("fvo_init_state",):
            getattr(lib, name).argtypes = [P]
        lib.fvo_set_state.argtypes = [P, P, P, P]
        lib.fvo_get_state.argtypes = [P, P, P, P]
        lib.fvo_set_scalars.argtypes = [P, C.c_double, C.c_double, C.c_int]
        lib.fvo_get_stats.argtypes = [P, C.POINTER(FvRunStats)]
        lib.fvo_run.argtypes = [P, C.c_int64, C.POINTER(FvRunStats)]
        lib.fvo_debug_step.argtypes = [P, C.c_int, P, P, P]
        lib.fvo_last_cfl.restype = C.c_double
        lib.fvo_last_cfl.argtypes = [P]
        lib.fvo_fvm_eval.argtypes = [C.c_int, P, P, C.c_int64]
        lib.fvo_set_weights.restype = C.c_int
        lib.fvo_set_weights.argtypes = [P, P, P, C.c_int]
        lib.fvo_last_dt.restype = C.c_double
        lib.fvo_last_dt.argtypes = [P]
        lib.fvo_schedule_loss.restype = C.c_int
        lib.fvo_schedule_loss.argtypes = [C.POINTER(FvParams), C.c_int, C.c_int, P, P, C.c_int, C.c_int64, P, P,
                                          P, P]
        lib.fvo_tlm_loss.restype = C.c_int
        lib.fvo_tlm_loss.argtypes = [C.POINTER(FvParams), C.c_int, C.c_int, P, P, C.c_int, C.c_int, P,
                                     C.c_int64, P, P, P, P, P]
        _oracle = lib
    return _oracle


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def _load_ref() -> C.CDLL:
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError(f"{REF_LIB} not built (needs the reference tree)")
        _ref = C.CDLL(REF_LIB)
    return _ref


def fvm_eval(fn: str, x) -> np.ndarray:
    """fv_math.h's float function `fn` (sin, cos, exp, tanh) on the host."""
    code = {"sin": 0, "cos": 1, "exp": 2, "tanh": 3}[fn]
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    _load_oracle().fvo_fvm_eval(code, _ptr(x), _ptr(y), x.size)
    return y


def set_threads(n: int) -> int:
    return _load_oracle().fvo_set_threads(int(n))


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class OracleSim:
    """One simulation of the CPU restatement, mirroring the C ABI's handle.

    math="libm": the apps' sin/exp/tanh from the host libm (the mode pinned
    to the reference build); math="fvm": from fv_math.h, as the library
    evaluates them (the mode the CUDA path is compared with bit for bit).
    """

    def __init__(self, params: FvParams, dtype=np.float32, math: str = "libm"):
        if math not in ("libm", "fvm"):
            raise ValueError("math must be 'libm' or 'fvm'")
        self.lib = _load_oracle()
        self.params = params.copy()
        self.dtype = np.dtype(dtype)
        self.math = math
        prec = self.dtype.itemsize
        self.h = self.lib.fvo_create(C.byref(self.params), prec, 1 if math == "fvm" else 0)
        if not self.h:
            raise ValueError("oracle rejected the parameters")
        self.shape = (params.ny, params.nx)

    def close(self):
        if self.h:
            self.lib.fvo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_state(self):
        self.lib.fvo_init_state(self.h)

    def set_state(self, u1, u2, u3):
        arrs = [np.ascontiguousarray(u, dtype=self.dtype).reshape(self.shape) for u in (u1, u2, u3)]
        self.lib.fvo_set_state(self.h, *[_ptr(a) for a in arrs])

    def get_state(self):
        out = [np.empty(self.shape, self.dtype) for _ in range(3)]
        self.lib.fvo_get_state(self.h, *[_ptr(a) for a in out])
        return out

    def set_scalars(self, dt, T, n=0):
        self.lib.fvo_set_scalars(self.h, float(dt), float(T), int(n))

    def set_weights(self, amp, phase):
        """Phased-array element amplitudes and phases."""
        a = np.ascontiguousarray(amp, np.float64)
        ph = np.ascontiguousarray(phase, np.float64)
        if self.lib.fvo_set_weights(self.h, _ptr(a), _ptr(ph), int(a.size)) != 0:
            raise ValueError("weights do not match the phased array")

    def stats(self) -> dict:
        st = FvRunStats()
        self.lib.fvo_get_stats(self.h, C.byref(st))
        return st.as_dict()

    def run(self, nsteps: int) -> dict:
        st = FvRunStats()
        rc = self.lib.fvo_run(self.h, int(nsteps), C.byref(st))
        d = st.as_dict()
        d["rc"] = rc
        return d

    def debug_step(self, stage: int):
        out = [np.empty(self.shape, self.dtype) for _ in range(3)]
        rc = self.lib.fvo_debug_step(self.h, int(stage), *[_ptr(a) for a in out])
        return rc, out

    def last_cfl(self) -> float:
        return self.lib.fvo_last_cfl(self.h)

    def last_dt(self) -> float:
        """dt of the attempt that the last run(1) accepted."""
        return self.lib.fvo_last_dt(self.h)

    def schedule(self, nsteps: int):
        """Run nsteps accepted steps one at a time; returns (dts, Ts): dt and
        T (before the step) of each accepted step, the schedule the
        library's adjoint holds fixed."""
        dts = np.empty(nsteps, np.float64)
        Ts = np.empty(nsteps, np.float64)
        for n in range(nsteps):
            Ts[n] = self.stats()["T"]
            st = self.run(1)
            if st["rc"] != 0:
                raise RuntimeError(f"oracle stopped with status {st['rc']} at step {n}")
            dts[n] = self.last_dt()
        return dts, Ts


def tlm_loss(params: FvParams, amp, phase, directions, dts, Ts, window, dtype=np.float64, math="fvm"):
    """The oracle's tangent-linear model of the phased array's windowed loss
    on a fixed dt schedule: (loss, d loss / d theta_r for each direction r).
    `directions` index the weights: k < nelem is amp[k], else phase[k -
    nelem] (at most 16). window = (i0, j0, ni, nj, first, last). dtype
    float32 runs the values along the FP32 oracle's trajectory, float64
    along the FP64 one; derivatives are double either way."""
    lib = _load_oracle()
    a = np.ascontiguousarray(amp, np.float64)
    ph = np.ascontiguousarray(phase, np.float64)
    d = np.ascontiguousarray(directions, np.int32)
    dts = np.ascontiguousarray(dts, np.float64)
    Ts = np.ascontiguousarray(Ts, np.float64)
    w = np.ascontiguousarray(window, np.int32)
    loss = np.zeros(1, np.float64)
    grad = np.zeros(len(d), np.float64)
    p = params.copy()
    rc = lib.fvo_tlm_loss(C.byref(p), np.dtype(dtype).itemsize, 1 if math == "fvm" else 0, _ptr(a), _ptr(ph),
                          int(a.size), int(d.size), _ptr(d), int(dts.size), _ptr(dts), _ptr(Ts), _ptr(w),
                          _ptr(loss), _ptr(grad))
    if rc != 0:
        raise RuntimeError(f"fvo_tlm_loss failed with status {rc}")
    return float(loss[0]), grad


def ref_call(params: FvParams, op: int, u, dtype=np.float32, nsteps: int = 0, scalars=None):
    """Call the reference shim: op 0 init, 1 run nsteps, 10+stage debug step.

    `u` is a list of three (ny, nx) arrays (updated in place); scalars is
    [dt, T, n, MDX, MDY] (updated in place). Returns (status, stats dict).
    """
    lib = _load_ref()
    key = REF_APP_KEYS[int(params.app)]
    suffix = "f32" if np.dtype(dtype) == np.float32 else "f64"
    fn = getattr(lib, f"fvref_{key}_{suffix}")
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(FvParams), C.c_int, C.c_int64, C.c_void_p, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.POINTER(FvRunStats)]
    if scalars is None:
        scalars = np.array([params.dtini, -params.tide, 0, 0, 0], np.float64)
    st = FvRunStats()
    p = params.copy()
    rc = fn(C.byref(p), int(op), int(nsteps), *[_ptr(a) for a in u], _ptr(scalars), C.byref(st))
    return rc, st.as_dict()


def schedule_loss(params: FvParams, amp, phase, dts, Ts, window, dtype=np.float64, math="fvm") -> float:
    """The phased array's windowed loss on a fixed dt schedule (tlm_loss's
    loss without derivatives): the evaluations of central differences."""
    lib = _load_oracle()
    a = np.ascontiguousarray(amp, np.float64)
    ph = np.ascontiguousarray(phase, np.float64)
    dts = np.ascontiguousarray(dts, np.float64)
    Ts = np.ascontiguousarray(Ts, np.float64)
    w = np.ascontiguousarray(window, np.int32)
    loss = np.zeros(1, np.float64)
    p = params.copy()
    rc = lib.fvo_schedule_loss(C.byref(p), np.dtype(dtype).itemsize, 1 if math == "fvm" else 0, _ptr(a), _ptr(ph),
                               int(a.size), int(dts.size), _ptr(dts), _ptr(Ts), _ptr(w), _ptr(loss))
    if rc != 0:
        raise RuntimeError(f"fvo_schedule_loss failed with status {rc}")
    return float(loss[0])
