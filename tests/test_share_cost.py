"""The step kernels' work distribution (fvgb::ShareCost in fv_internal.h),
compiled for the host from the same header: the warps' cost shares tile
every (window, row) position once for many grid shapes and warp counts,
and the windows it weights as having ghost columns are exactly those of
the step kernel's edge test. Runs on the CPU (g++)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_share_cost_tiles_every_window_row_once(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "share_cost_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "fivonagi_gb300", "csrc"), "-o", exe,
                    os.path.join(ROOT, "tests", "native", "share_cost_check.cpp")], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().startswith("share_cost ok"), out.stdout
