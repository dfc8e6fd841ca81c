"""The C ABI from a plain C program (tests/native/c_driver.c).

The reference's host code becomes a C program against include/fivonagi.h:
parameters, initial values, the calcFrame loop to each print time, the
state copied back, and per-step stats through the pipelined calls. On CPU
the program must compile and link as C99 with gcc against the header and
the library; on the GPU its final state must equal the Python binding's
run of the same steps bit for bit.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from fivonagi_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "native", "c_driver.c")


def _build(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip("library not built")
    exe = str(tmp_path / "c_driver")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
                    "-L", _abi.LIB_DIR, "-lfivonagi", f"-Wl,-rpath,{_abi.LIB_DIR}", "-o", exe], check=True)
    return exe


def test_c_driver_builds_as_c99_against_the_header_and_library(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_c_driver_matches_the_python_binding(tmp_path):
    from fivonagi_gb300 import Simulation

    exe = _build(tmp_path)
    nx, ny, nprint, dtprint, npipe = 128, 96, 18, 1.0, 10  # past T = 0, where the source starts (TIDE = 15)
    out = tmp_path / "u.bin"
    r = subprocess.run([exe, str(nx), str(ny), str(nprint), str(dtprint), str(npipe), str(out)],
                       capture_output=True, text=True, check=True)
    T, n, accepted, rejected = r.stdout.split()
    u = np.fromfile(out, np.float32).reshape(3, ny, nx)
    p = _abi.default_params("hifu-beam").replace(nx=nx, ny=ny, xmax=(nx - 1) / 16.0, ymax=(ny - 1) / 16.0)
    sim = Simulation(p)
    sim.init_state()
    tprint = -p.tide + dtprint
    for _ in range(nprint):
        sim.run_until(tprint)
        tprint += dtprint
    stats = list(sim.steps_pipelined(npipe, block=1))
    g = sim.get_state()
    st = sim.stats()
    sim.close()
    assert int(n) == st["n"] > 0 and np.float32(float(T)) == np.float32(st["T"])
    assert int(rejected) >= 0 and int(accepted) >= sum(s["accepted"] for s in stats)
    for f in range(3):
        np.testing.assert_array_equal(u[f], g[f])
    assert np.abs(u[0]).max() > 0  # the source has driven the medium
