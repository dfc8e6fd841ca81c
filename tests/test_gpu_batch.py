"""Batches: every simulation of an uneven batch stepped by one launch must
reproduce, bit for bit, the oracle run of that simulation alone."""
import numpy as np
import pytest

from fivonagi_gb300 import Batch, Simulation, _abi, configs
from oracle.oracle import OracleSim
from tests.helpers import perturbed, rel_l2, same_values, small_params

pytestmark = pytest.mark.gpu

MIXED = [(2, 64, 32), (0, 100, 37), (1, 27, 61), (3, 300, 130), (2, 8, 8), (3, 130, 64)]


def _states(plist, seed=5):
    out = []
    for k, p in enumerate(plist):
        o = OracleSim(p, np.float32, math="fvm")
        o.init_state()
        out.append(perturbed(o.get_state(), seed + k, 1e-4))
    return out


def test_mixed_batch_matches_each_simulation_alone():
    plist = [small_params(app, nx, ny) for app, nx, ny in MIXED]
    u0 = _states(plist)
    b = Batch(plist)
    for k, u in enumerate(u0):
        b.set_state(k, *u)
    st = b.run(70)
    for k, p in enumerate(plist):
        o = OracleSim(p, np.float32, math="fvm")
        o.set_state(*u0[k])
        so = o.run(70)
        assert st[k]["accepted"] == 70 and st[k]["rejected"] == so["rejected"]
        assert np.float32(st[k]["T"]) == np.float32(so["T"])
        g, r = b.get_state(k), o.get_state()
        for f in range(3):
            assert same_values(g[f], r[f]), f"simulation {k} field {f}: rel L2 {rel_l2(g[f], r[f]):.3e}"
    b.close()


def test_batch_equals_plain_path():
    plist = [small_params(3, 200, 96), small_params(2, 96, 200)]
    u0 = _states(plist, seed=11)
    b = Batch(plist)
    for k, u in enumerate(u0):
        b.set_state(k, *u)
    b.run(40)
    for k, p in enumerate(plist):
        s = Simulation(p)
        s.set_state(*u0[k])
        s.run(40)
        g, r = b.get_state(k), s.get_state()
        assert all(same_values(g[f], r[f]) for f in range(3))
        s.close()
    b.close()


def test_one_simulation_retries_while_the_others_step():
    plist = [small_params(2, 64, 32).replace(dtini=0.3), small_params(2, 64, 32), small_params(0, 64, 32)]
    u0 = _states(plist, seed=2)
    b = Batch(plist)
    for k, u in enumerate(u0):
        b.set_state(k, *u)
    st = b.run(12)
    for k, p in enumerate(plist):
        o = OracleSim(p, np.float32, math="fvm")
        o.set_state(*u0[k])
        so = o.run(12)
        assert st[k]["rejected"] == so["rejected"] and st[k]["accepted"] == 12
        g, r = b.get_state(k), o.get_state()
        assert all(same_values(g[f], r[f]) for f in range(3))
    assert st[0]["rejected"] >= 1 and st[1]["rejected"] == 0
    b.close()


def test_a_failing_simulation_does_not_stop_the_others():
    plist = [small_params(2, 64, 32), small_params(2, 64, 32)]
    u0 = _states(plist, seed=3)
    bad = [x.copy() for x in u0[1]]
    bad[0][10:20, 10:20] = -0.9
    b = Batch(plist)
    b.set_state(0, *u0[0])
    b.set_state(1, *bad)
    rc, st = b.run_status(20)
    assert rc == _abi.FV_NEGATIVE_EIGENVALUE
    assert st[1]["status"] == _abi.FV_NEGATIVE_EIGENVALUE and st[0]["status"] == 0
    assert st[0]["accepted"] == 20
    o = OracleSim(plist[0], np.float32, math="fvm")
    o.set_state(*u0[0])
    o.run(20)
    g, r = b.get_state(0), o.get_state()
    assert all(same_values(g[f], r[f]) for f in range(3))
    b.close()



def test_config3_instances_equal_the_plain_path():
    """A dozen simulations from the batched workload's generator (sides from
    256 to 2048, random beta, dissipation, amplitude and wavelength), at the
    batch's default launch (eight waves of CTAs), against each simulation
    run alone on the plain path (itself checked against the oracle)."""
    plist = configs.batched(12, seed=3)
    b = Batch(plist)
    b.init_state()
    st = b.run(30)
    for k, p in enumerate(plist):
        s = Simulation(p)
        s.init_state()
        ss = s.run(30)
        assert st[k]["accepted"] == 30 and st[k]["rejected"] == ss["rejected"]
        assert np.float32(st[k]["T"]) == np.float32(ss["T"])
        g, r = b.get_state(k), s.get_state()
        for f in range(3):
            assert same_values(g[f], r[f]), f"simulation {k} ({p.nx}x{p.ny}) field {f}"
        s.close()
    b.close()


def test_supersonic_instance_matches_oracle():
    """The batch kernel's subsonic solve flags an instance's supersonic
    interfaces for the batch fix-up pass: one step of patches moving at 0.9
    is the oracle's bit for bit, beside an ordinary instance."""
    plist = [small_params(2, 96, 48), small_params(0, 64, 32)]
    u0 = _states(plist, seed=21)
    u0[0][1][10:22, 20:40] += np.float32(0.9)
    u0[0][2][26:40, 50:70] -= np.float32(0.9)
    b = Batch(plist)
    for k, u in enumerate(u0):
        b.set_state(k, *u)
    st = b.run(1)
    for k, p in enumerate(plist):
        o = OracleSim(p, np.float32, math="fvm")
        o.set_state(*u0[k])
        so = o.run(1)
        assert so["rc"] == 0 and st[k]["accepted"] == 1 and st[k]["rejected"] == so["rejected"]
        g, r = b.get_state(k), o.get_state()
        for f in range(3):
            assert same_values(g[f], r[f]), f"simulation {k} field {f}: rel L2 {rel_l2(g[f], r[f]):.3e}"
    b.close()


@pytest.mark.parametrize("blocks", [1, 2, 5])
def test_few_ctas_batch_matches_oracle(blocks):
    """A batch launched with 1-5 CTAs: each warp's share spans several
    simulations and windows; every simulation is still the oracle's bit for
    bit."""
    plist = [small_params(app, nx, ny) for app, nx, ny in MIXED]
    u0 = _states(plist, seed=31)
    b = Batch(plist)
    b.set_launch(blocks)
    for k, u in enumerate(u0):
        b.set_state(k, *u)
    st = b.run(10)
    for k, p in enumerate(plist):
        o = OracleSim(p, np.float32, math="fvm")
        o.set_state(*u0[k])
        so = o.run(10)
        assert st[k]["accepted"] == 10 and st[k]["rejected"] == so["rejected"]
        g, r = b.get_state(k), o.get_state()
        for f in range(3):
            assert same_values(g[f], r[f]), f"simulation {k} field {f}: rel L2 {rel_l2(g[f], r[f]):.3e}"
    b.close()
