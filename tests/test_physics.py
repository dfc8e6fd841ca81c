"""Physics-level known answer: the taylor-angle-xy app's analytic profile.

The app drives a plane wave whose steady shape is the Taylor solution
u1 = ISPRHOA tanh(ISPC (x cos(angle) + y sin(angle) - T))
(apps/taylor-angle-xy/boundary.h:10-56, data_collect.h:37-96), with
ISPRHOA = -DIFFDELTA / BETA; the reference measures the numeric profile
against it along an oblique cut with relative L1, L2 and L-infinity norms
(data_export.h:111-127; fivonagi_gb300.export.taylor_cut / error_norms).

At the app's own parameters (DIFFDELTA 1e-7, so an amplitude of 1e-7) FP32
cannot hold the wave: rho = 1 + u1 keeps about one significant digit of
it, in the reference's FP32 evaluation and here alike. The FP64 oracle
follows the analytic profile; with DIFFDELTA and ISPRHOA scaled together
(same shock width, amplitude 1e-3) the FP32 evaluation -- which the GPU
reproduces bit for bit -- follows it as closely as FP64 does.
"""
import numpy as np
import pytest

from fivonagi_gb300 import _abi
from fivonagi_gb300.export import error_norms, taylor_cut
from oracle import oracle
from oracle.oracle import OracleSim

# relative L2 of the cut against the analytic profile at T ~ 15 (measured
# 1.7e-2 to 1.9e-2 on the app's 64 x 64 grid)
L2_BAR = 2.5e-2


def taylor_params(scale: float = 1.0, angle: float = 0.0):
    p = _abi.default_params("taylor-angle-xy")
    return p.replace(diffdelta=p.diffdelta * scale, isp_rhoa=p.isp_rhoa * scale, angle=angle)


def _oracle_error(p, dtype, T_end):
    o = OracleSim(p, dtype, math="libm")
    o.init_state()
    while o.stats()["T"] < T_end:
        assert o.run(10)["rc"] == 0
    s = o.stats()
    num, ana = taylor_cut(np.asarray(o.get_state()[0]), p, s["T"], s["mdx"], s["mdy"])
    o.close()
    assert len(num) > 30 and s["mdx"] > 0  # the window has followed the wave
    return error_norms(num, ana)


@pytest.mark.parametrize("angle", [0.0, 0.5])
def test_fp64_oracle_follows_the_analytic_profile(angle):
    oracle.set_threads(2)
    l1, l2, linf = _oracle_error(taylor_params(1.0, angle), np.float64, 15.0)
    assert l2 <= L2_BAR and l1 <= l2 and linf < 0.15, (l1, l2, linf)


def test_fp32_follows_it_at_a_resolvable_amplitude_and_not_at_1e_7():
    oracle.set_threads(2)
    l2_64 = _oracle_error(taylor_params(1e4), np.float64, 15.0)[1]
    l2_32 = _oracle_error(taylor_params(1e4), np.float32, 15.0)[1]
    assert l2_32 <= L2_BAR and abs(l2_32 - l2_64) <= 0.05 * l2_64, (l2_32, l2_64)
    assert _oracle_error(taylor_params(1.0), np.float32, 15.0)[1] > 0.3  # FP32 rounding, not physics
