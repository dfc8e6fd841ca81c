"""Bit-for-bit parity with the oracle at the headline size.

The focused beam on 4096 x 2048 cells (the plain method at full size, the
bench's workload), started from a seeded perturbation of its initial state
so that every cell of the grid does the full arithmetic (waves, limiters,
diffusion, the CFL reduction over all 8.4 M cells), with each division
mode of the step kernel. A few steps keep the oracle's share to seconds on
the host's cores.
"""
import os
import sys

import numpy as np
import pytest

from fivonagi_gb300 import Simulation, _abi
from oracle import oracle
from oracle.oracle import OracleSim
from tests.helpers import perturbed, rel_l2, same_values

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("division", [_abi.FV_DIVISION_EXACT, _abi.FV_DIVISION_FMA])
def test_headline_size_matches_oracle(division):
    import bench

    p = bench.workload_params(True)
    assert (p.nx, p.ny) == (4096, 2048)
    oracle.set_threads(os.cpu_count() or 1)
    orc = OracleSim(p, np.float32, math="fvm")
    orc.init_state()
    u = perturbed(orc.get_state(), 7, 1e-4)
    orc.set_state(*u)
    sim = Simulation(p)
    sim.set_division(division)
    sim.set_state(*u)
    n = 6
    sg = sim.run(n)
    so = orc.run(n)
    assert so["rc"] == 0
    assert sg["accepted"] == n and so["accepted"] == n
    assert sg["rejected"] == so["rejected"]
    g, o = sim.get_state(), orc.get_state()
    for f in range(3):
        assert same_values(g[f], o[f]), f"field {f}: rel L2 {rel_l2(g[f], o[f]):.3e}"
    assert np.float32(sg["dt"]) == np.float32(so["dt"])
    assert np.float32(sg["T"]) == np.float32(so["T"])
    sim.close()
    orc.close()
