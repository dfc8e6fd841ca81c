"""ctypes mirror of include/fivonagi.h and the loader of libfivonagi.so.

The library is the product: a C ABI over hand-written sm_103a kernels. This
module only declares its types and entry points; it never computes anything
itself, and loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libfivonagi.so")

# fv_status (include/fivonagi.h)
FV_OK = 0
FV_DT_TOO_LARGE = 1
FV_NEGATIVE_EIGENVALUE = 2
FV_TRANSONIC = 3
FV_COLLECT_OVERFLOW = 4
FV_TIMEOUT = 5
FV_CUDA_ERROR = 6
FV_BAD_ARG = 7
FV_NO_DEVICE = 8

STATUS_NAMES = {
    FV_OK: "ok",
    FV_DT_TOO_LARGE: "dt too large",
    FV_NEGATIVE_EIGENVALUE: "negative eigenvalue",
    FV_TRANSONIC: "transonic rarefaction",
    FV_COLLECT_OVERFLOW: "data collection overflow",
    FV_TIMEOUT: "device wait timed out",
    FV_CUDA_ERROR: "CUDA error",
    FV_BAD_ARG: "bad argument",
    FV_NO_DEVICE: "no usable device",
}

# fv_app
FV_APP_HIFU_BEAM = 0
FV_APP_TAYLOR_ANGLE_XY = 1
FV_APP_PLANE_WAVE = 2
FV_APP_FOCUSED_BEAM = 3
FV_APP_PHASED_ARRAY = 4

# CTA shapes of the step kernel (fv_set_cta_shape): warps per CTA x CTAs per SM
FV_CTA_SHAPES = {0: "4x4", 1: "2x8", 2: "1x16", 3: "1x18", 4: "4x4/ahead1", 5: "4x4/ahead3"}

# division in the step kernel (fv_set_division)
FV_DIVISION_DEFAULT = -1
FV_DIVISION_FMA = 0
FV_DIVISION_EXACT = 1
APP_NAMES = {
    "hifu-beam": FV_APP_HIFU_BEAM,
    "taylor-angle-xy": FV_APP_TAYLOR_ANGLE_XY,
    "plane-wave": FV_APP_PLANE_WAVE,
    "focused-beam": FV_APP_FOCUSED_BEAM,
    "phased-array": FV_APP_PHASED_ARRAY,
}

# fv_stage
FV_STAGE_BOUNDARY = 0
FV_STAGE_SWEEP_Y = 1
FV_STAGE_SWEEP_X = 2
FV_STAGE_SOURCE = 3


class FvParams(C.Structure):
    _fields_ = [
        ("app", C.c_int32),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("cfl_even_only", C.c_int32),
        ("moving_domain", C.c_int32),
        ("exact", C.c_int32),
        ("max_retries", C.c_int32),
        ("array_elems", C.c_int32),
        ("xmax", C.c_double),
        ("ymax", C.c_double),
        ("beta", C.c_double),
        ("diffdelta", C.c_double),
        ("cflmax", C.c_double),
        ("cflwhish", C.c_double),
        ("dtini", C.c_double),
        ("tide", C.c_double),
        ("mdvx", C.c_double),
        ("mdvy", C.c_double),
        ("mdt", C.c_double),
        ("ampl", C.c_double),
        ("frec", C.c_double),
        ("angle", C.c_double),
        ("isp_a", C.c_double),
        ("isp_f", C.c_double),
        ("isp_rhoa", C.c_double),
        ("isp_c", C.c_double),
        ("aperture", C.c_double),
        ("center", C.c_double),
        ("ramp_periods", C.c_double),
    ]

    def copy(self) -> "FvParams":
        out = FvParams()
        C.pointer(out)[0] = self
        return out

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}

    def replace(self, **kw) -> "FvParams":
        out = self.copy()
        for k, v in kw.items():
            if not hasattr(out, k):
                raise AttributeError(f"fv_params has no field {k!r}")
            setattr(out, k, v)
        return out


class FvRunStats(C.Structure):
    _fields_ = [
        ("accepted", C.c_int64),
        ("rejected", C.c_int64),
        ("dt", C.c_double),
        ("T", C.c_double),
        ("cfl", C.c_double),
        ("n", C.c_int32),
        ("status", C.c_int32),
        ("mdx", C.c_int32),
        ("mdy", C.c_int32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class FvLossWindow(C.Structure):
    _fields_ = [
        ("i0", C.c_int32),
        ("j0", C.c_int32),
        ("ni", C.c_int32),
        ("nj", C.c_int32),
        ("step_first", C.c_int64),
        ("step_last", C.c_int64),
    ]


class FvCollectSpec(C.Structure):
    _fields_ = [
        ("nprobes", C.c_int32),
        ("probe_i", C.c_int32 * 8),
        ("probe_j", C.c_int32 * 8),
        ("envelope_row", C.c_int32),
        ("envelope_len", C.c_int32),
        ("capacity", C.c_int32),
        ("envelope_halfwidth", C.c_double),
    ]


class FvRenderSpec(C.Structure):
    _fields_ = [
        ("i0", C.c_int32),
        ("j0", C.c_int32),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("zoom", C.c_int32),
        ("jcut", C.c_int32),
        ("overlays", C.c_int32),
        ("reserved", C.c_int32),
        ("plot_scale", C.c_double),
    ]


class FvStepResult(C.Structure):
    _fields_ = [
        ("accepted", C.c_int32),
        ("status", C.c_int32),
        ("cfl", C.c_double),
        ("dt_next", C.c_double),
        ("T", C.c_double),
        ("mdx", C.c_int32),
        ("mdy", C.c_int32),
    ]


_P = C.c_void_p
_FP = C.POINTER(C.c_float)

# name -> (restype, argtypes); every entry point declared in include/fivonagi.h
PROTOTYPES = {
    "fv_version": (C.c_char_p, []),
    "fv_last_error_string": (C.c_char_p, []),
    "fv_default_params": (C.c_int, [C.c_int32, C.POINTER(FvParams)]),
    "fv_create": (C.c_int, [C.POINTER(FvParams), C.POINTER(_P)]),
    "fv_destroy": (C.c_int, [_P]),
    "fv_init_state": (C.c_int, [_P]),
    "fv_set_state": (C.c_int, [_P, _P, _P, _P, C.c_int32]),
    "fv_get_state": (C.c_int, [_P, _P, _P, _P, C.c_int32]),
    "fv_set_scalars": (C.c_int, [_P, C.c_double, C.c_double, C.c_int32]),
    "fv_get_stats": (C.c_int, [_P, C.POINTER(FvRunStats)]),
    "fv_set_array_weights": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32]),
    "fv_adjoint_create": (C.c_int, [C.POINTER(FvParams), C.POINTER(FvLossWindow), C.c_int64, C.c_int32,
                                    C.POINTER(_P)]),
    "fv_adjoint_destroy": (C.c_int, [_P]),
    "fv_adjoint_set_stream": (C.c_int, [_P, _P]),
    "fv_adjoint_forward": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "fv_adjoint_backward": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fv_adjoint_replay": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "fv_adjoint_schedule": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fv_adjoint_get_state": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "fv_adjoint_batch_create": (C.c_int, [C.POINTER(FvParams), C.c_int32, C.POINTER(FvLossWindow), C.c_int64,
                                          C.c_int32, C.POINTER(_P)]),
    "fv_adjoint_batch_destroy": (C.c_int, [_P]),
    "fv_adjoint_batch_set_stream": (C.c_int, [_P, _P]),
    "fv_adjoint_batch_forward": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "fv_adjoint_batch_backward": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fv_adjoint_batch_schedule": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fv_filter_u1": (C.c_int, [_P, C.c_double, _P, C.c_int32]),
    "fv_render": (C.c_int, [_P, C.POINTER(FvRenderSpec), _P, C.c_int32]),
    "fv_collect_enable": (C.c_int, [_P, C.POINTER(FvCollectSpec)]),
    "fv_collect_read": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                  C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "fv_snapshot": (C.c_int, [_P]),
    "fv_restore": (C.c_int, [_P]),
    "fv_set_stream": (C.c_int, [_P, _P]),
    "fv_run": (C.c_int, [_P, C.c_int64, C.POINTER(FvRunStats)]),
    "fv_run_until": (C.c_int, [_P, C.c_double, C.POINTER(FvRunStats)]),
    "fv_launch_attempts": (C.c_int, [_P, C.c_int64]),
    "fv_time_attempts": (C.c_int, [_P, C.c_int32, _P, _P]),
    "fv_time_run": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_float)]),
    "fv_device_name": (C.c_int, [C.c_char_p, C.c_int32]),
    "fv_set_division": (C.c_int, [_P, C.c_int32]),
    "fv_get_division": (C.c_int, [_P, _P]),
    "fv_sync": (C.c_int, [_P, C.POINTER(FvRunStats)]),
    "fv_steps_async": (C.c_int, [_P, C.c_int32]),
    "fv_step_wait": (C.c_int, [_P, C.POINTER(FvRunStats)]),
    "fv_debug_step": (C.c_int, [_P, C.c_int32, _P, _P, _P]),
    "fv_set_launch": (C.c_int, [_P, C.c_int32]),
    "fv_set_cta_shape": (C.c_int, [_P, C.c_int32]),
    "fv_get_cta_shape": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "fv_get_launch": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "fv_batch_create": (C.c_int, [C.c_int32, C.POINTER(FvParams), C.POINTER(_P)]),
    "fv_batch_destroy": (C.c_int, [_P]),
    "fv_batch_set_stream": (C.c_int, [_P, _P]),
    "fv_batch_init_state": (C.c_int, [_P]),
    "fv_batch_set_state": (C.c_int, [_P, C.c_int32, _P, _P, _P, C.c_int32]),
    "fv_batch_get_state": (C.c_int, [_P, C.c_int32, _P, _P, _P, C.c_int32]),
    "fv_batch_run": (C.c_int, [_P, C.c_int64, C.POINTER(FvRunStats)]),
    "fv_batch_launch_attempts": (C.c_int, [_P, C.c_int64]),
    "fv_batch_sync": (C.c_int, [_P, C.POINTER(FvRunStats)]),
    "fv_batch_time_run": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_float)]),
    "fv_batch_set_launch": (C.c_int, [_P, C.c_int32]),
    "fv_batch_get_launch": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "fv_step_noalloc": (C.c_int, [C.POINTER(FvParams), _P, _P, _P, _P, _P, _P, C.c_double, C.c_double,
                                  C.c_int32, C.c_int32, _P, C.POINTER(FvStepResult)]),
}

_lib = None


class FvError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        name = STATUS_NAMES.get(status, f"status {status}")
        msg = f"{where}: {name}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


def load_library(path: str | None = None) -> C.CDLL:
    """Load libfivonagi.so and declare its prototypes.

    Raises FileNotFoundError when the library is missing: there is no
    fallback path.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
        )
    lib = C.CDLL(p)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int, where: str) -> None:
    if status != FV_OK:
        detail = ""
        if _lib is not None:
            raw = _lib.fv_last_error_string()
            detail = raw.decode() if raw else ""
        raise FvError(status, where, detail)


def default_params(app: int | str) -> FvParams:
    """The app's reference parameter values (its parameters.h), from the library."""
    if isinstance(app, str):
        app = APP_NAMES[app]
    lib = load_library()
    p = FvParams()
    check(lib.fv_default_params(app, C.byref(p)), "fv_default_params")
    return p


def device_name() -> str:
    """The current CUDA device's name, from the library."""
    lib = load_library()
    buf = C.create_string_buffer(256)
    check(lib.fv_device_name(buf, len(buf)), "fv_device_name")
    return buf.value.decode()
