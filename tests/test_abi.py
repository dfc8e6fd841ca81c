"""The C ABI of libfivonagi.so without a GPU: symbols, layout, defaults, errors."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from fivonagi_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fivonagi.h")


def _declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(fv_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_function():
    lib = _abi.load_library()
    names = _declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
        assert name in _abi.PROTOTYPES, f"{name} has no ctypes prototype"


def test_struct_layout_matches_header(tmp_path):
    """Offsets of fv_params / fv_run_stats as gcc lays them out, vs ctypes."""
    src = tmp_path / "layout.c"
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for struct, cls in (("fv_params", _abi.FvParams), ("fv_run_stats", _abi.FvRunStats)):
        lines.append(f'printf("{struct} %zu\\n", sizeof({struct}));')
        for name, _ in cls._fields_:
            lines.append(f'printf("{struct}.{name} %zu\\n", offsetof({struct}, {name}));')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(ln.split() for ln in out if ln.strip())
    for struct, cls in (("fv_params", _abi.FvParams), ("fv_run_stats", _abi.FvRunStats)):
        assert int(got[struct]) == C.sizeof(cls)
        for name, _ in cls._fields_:
            assert int(got[f"{struct}.{name}"]) == getattr(cls, name).offset, f"{struct}.{name}"


def _f32(x):
    return np.float32(x)


def test_hifu_defaults_follow_its_parameters_h():
    """apps/hifu-beam/parameters.h with ETAC=1, CFLW=90, ISPAM=30, evaluated in FP32."""
    p = _abi.default_params("hifu-beam")
    NX, NY = 512, 1024
    XMAX, YMAX, FREC = _f32(25.0), _f32(50.0), _f32(1.0)
    PI = _f32(3.1415926)
    ISPW = _f32(2) * PI * FREC
    ISPlambda = _f32(2) * PI / ISPW
    ISPa = _f32(30) * ISPlambda
    ISPF = _f32(50.0 * float(ISPlambda) / float(XMAX / _f32(NX - 1)))
    dxf, dyf = float(XMAX / _f32(NX - 1)), float(YMAX / _f32(NY - 1))
    TIDE = np.floor(float(_f32(2) + _f32(4) / FREC) +
                    float(ISPa * ISPa * _f32(dxf)) / (2.0 * float(ISPF) * dyf * dyf))
    assert (p.nx, p.ny) == (NX, NY)
    assert p.xmax == 25.0 and p.ymax == 50.0
    assert p.isp_a == float(ISPa) and p.isp_f == float(ISPF) and p.tide == TIDE == 15.0
    assert np.float32(p.beta) == _f32(4.8) and np.float32(p.diffdelta) == _f32(0.0002974)
    assert np.float32(p.cflwhish) == _f32(0.9) and p.mdt == 12.5 and p.moving_domain == 1


def test_taylor_defaults_follow_its_parameters_h():
    p = _abi.default_params("taylor-angle-xy")
    assert (p.nx, p.ny) == (64, 64)
    assert p.mdt == 6.25 and p.tide == 4.0
    assert np.float32(p.isp_rhoa) == _f32(-_f32(1e-7) / _f32(1.0))
    assert np.float32(p.isp_c) == _f32(2.1972245773362196)


def test_workload_defaults():
    pw = _abi.default_params("plane-wave")
    assert (pw.nx, pw.ny) == (512, 512) and pw.xmax == 511 / 16 and abs(pw.angle - np.pi / 6) < 1e-15
    fb = _abi.default_params("focused-beam")
    assert (fb.nx, fb.ny) == (4096, 2048) and fb.xmax == 4095 / 24
    assert fb.aperture == 1024 and fb.center == 1024 and fb.isp_f == 3000 and fb.ramp_periods == 5
    pa = _abi.default_params("phased-array")
    assert (pa.nx, pa.ny, pa.array_elems) == (1024, 1024, 128) and pa.aperture / pa.array_elems == 8


def test_bad_arguments_are_rejected_before_any_device_work():
    lib = _abi.load_library()
    h = C.c_void_p()
    p = _abi.default_params("plane-wave")
    for bad in (p.replace(nx=4), p.replace(ny=7), p.replace(nx=65536, ny=32768),  # below 8x8, above 2^30 cells
                p.replace(app=9), p.replace(xmax=-1.0), p.replace(dtini=0.0),
                p.replace(cflmax=0.0), p.replace(cflwhish=-1.0),
                _abi.default_params("focused-beam").replace(ramp_periods=0.0),
                _abi.default_params("phased-array").replace(array_elems=0),
                _abi.default_params("phased-array").replace(array_elems=100)):
        assert lib.fv_create(C.byref(bad), C.byref(h)) == _abi.FV_BAD_ARG
        assert lib.fv_last_error_string()
    assert lib.fv_create(None, C.byref(h)) == _abi.FV_BAD_ARG
    assert lib.fv_default_params(42, C.byref(p)) == _abi.FV_BAD_ARG
    assert lib.fv_destroy(None) == _abi.FV_OK
    assert lib.fv_run(None, 1, None) == _abi.FV_BAD_ARG
    assert lib.fv_steps_async(None, 1) == _abi.FV_BAD_ARG
    assert lib.fv_step_wait(None, None) == _abi.FV_BAD_ARG


def test_no_device_is_a_status_not_a_crash():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _abi.load_library()
    h = C.c_void_p()
    p = _abi.default_params("plane-wave")
    assert lib.fv_create(C.byref(p), C.byref(h)) == _abi.FV_NO_DEVICE
    with pytest.raises(_abi.FvError):
        from fivonagi_gb300 import Simulation
        Simulation(p)


def test_restore_without_snapshot_is_bad_arg_without_device():
    # no device here: fv_create fails first; the argument check on a NULL
    # handle needs no device
    lib = _abi.load_library()
    assert lib.fv_restore(None) == _abi.FV_BAD_ARG
    assert lib.fv_snapshot(None) == _abi.FV_BAD_ARG


def test_adjoint_rejects_null_arguments_without_device():
    lib = _abi.load_library()
    assert lib.fv_adjoint_create(None, None, 10, 0, None) == _abi.FV_BAD_ARG
    assert lib.fv_adjoint_backward(None, None, None) == _abi.FV_BAD_ARG
    assert lib.fv_adjoint_destroy(None) == _abi.FV_OK
