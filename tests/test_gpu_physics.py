"""The GPU solver against the taylor-angle-xy app's analytic profile.

At an amplitude FP32 can hold (DIFFDELTA and ISPRHOA scaled together by
1e4, the same shock width as the app's own parameters), the GPU's profile
along the reference's oblique cut follows the analytic Taylor solution to
within L2_BAR relative L2 at T ~ 15, as the FP64 oracle does
(tests/test_physics.py), at both a planar and an oblique angle, with the
moving window following the wave.
"""
import pytest

from fivonagi_gb300 import Simulation
from fivonagi_gb300.export import error_norms, taylor_cut
from tests.test_physics import L2_BAR, taylor_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("angle", [0.0, 0.5])
def test_gpu_follows_the_analytic_profile(angle):
    p = taylor_params(1e4, angle)
    sim = Simulation(p)
    sim.init_state()
    st = sim.run_until(15.0)
    num, ana = taylor_cut(sim.get_state()[0], p, st["T"], st["mdx"], st["mdy"])
    sim.close()
    assert st["mdx"] > 0 and len(num) > 30
    l1, l2, linf = error_norms(num, ana)
    print(f"angle {angle}: T {st['T']:.3f}, GPU FP32 vs analytic L1 {l1:.3e} L2 {l2:.3e} Linf {linf:.3e}")
    assert l2 <= L2_BAR and l1 <= l2 and linf < 0.15, (l1, l2, linf)
