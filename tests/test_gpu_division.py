"""The step kernel's FMA division against the GPU's IEEE division.

The step kernel divides with Markstein's FMA sequence (fvgb::DivFma in
fv_device.cuh) and leaves the rows where an operand falls outside the range
in which that sequence is proven to round correctly to a recomputation with
exact division (fvgb::DivExact). This test builds tests/native/division_probe.cu against
the same header and runs it: an exhaustive check of the reciprocal for
every divisor in range, and sampled quotients around every bound of the
safety check; every quotient the check lets through must equal the IEEE
quotient bit for bit.
"""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    pytest.fail("nvcc not found")


def test_fma_division_is_ieee_where_not_flagged(tmp_path):
    exe = str(tmp_path / "division_probe")
    subprocess.run([_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I", os.path.join(ROOT, "fivonagi_gb300", "csrc"), "-o", exe,
                    os.path.join(ROOT, "tests", "native", "division_probe.cu")], check=True)
    out = subprocess.run([exe, "200000000"], capture_output=True, text=True, timeout=600)
    rows = {}
    for line in out.stdout.splitlines():
        f = line.split()
        if len(f) >= 4 and f[1].isdigit():
            rows[f[0]] = (int(f[1]), int(f[2]), int(f[3]), line)
    assert out.returncode == 0, out.stdout + out.stderr
    assert rows["recip_all"][0] == 151 << 24 and rows["recip_all"][2] == 0
    for name, (n, flagged, bad, line) in rows.items():
        assert bad == 0, line
        assert flagged <= n
    # the solver's own magnitudes, the tails' divisors and zero dividends
    # never need the IEEE recomputation
    assert rows["solver_like"][1] == 0
    assert rows["tail_divisors"][1] == 0
    assert rows["zero_dividend"][1] < rows["zero_dividend"][0]
    # powers of two within the divisor range take any dividend
    assert rows["pow2_divisor"][1] < rows["pow2_divisor"][0] // 2
    # the fix-up pass's exact division: checked on every class, and it
    # flags nothing in the classes the solver produces, tiny and subnormal
    # dividends included
    assert sum(1 for k in rows if k.startswith("xdiv_")) == 15
    # the normal-quotient division: checked on every class (bad == 0 above);
    # it flags nothing where the solver's quotients are normal
    assert sum(1 for k in rows if k.startswith("ndiv_")) == 15
    for name in ("solver_like", "dividend_2^-100", "exact_quotients"):
        assert rows["ndiv_" + name][1] == 0, rows["ndiv_" + name][3]
    # zero and subnormal divisors reach the scaled-dividend divisions with
    # no range test of their own: the NaN reciprocal flags them (bad == 0
    # above), while divisors of 2^-126 .. 2^-124 pass unflagged
    for pre in ("xdiv_", "ndiv_"):
        n, flagged, _, line = rows[pre + "divisor_below_2^-124"]
        assert 0 < flagged < n, line
    for name in ("solver_like", "tiny_dividend", "subnormal_dividend",
                 "dividend_2^-100", "tail_divisors", "exact_quotients"):
        assert rows["xdiv_" + name][1] == 0, rows["xdiv_" + name][3]
    # the limiter's ratio: flagged only for tiny dividends over unscaled
    # divisors (a small share of these synthetic products of waves)
    assert rows["ratio_waves"][1] < rows["ratio_waves"][0] // 4
    for name in ("ratio_wide", "ratio_mid", "ratio_waves"):
        assert rows[name][2] == 0
