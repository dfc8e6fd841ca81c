"""On-device data collection against the oracle, step by step."""
import numpy as np
import pytest

from fivonagi_gb300 import Simulation, _abi
from oracle.oracle import OracleSim
from tests.helpers import small_params

pytestmark = pytest.mark.gpu


def test_collection_matches_oracle_with_moving_window():
    # hifu hooks with the window moving from T = 0.5, so probes, envelope and
    # lab coordinates all move
    p = small_params(0, 96, 48).replace(moving_domain=1, mdt=0.5, mdvx=1.0, mdvy=0.0)
    probes = [(20, 2), (40, 2), (55, 10), (3, 2)]  # the last one leaves the window
    nsteps, env_len = 120, 4 * p.nx
    sim = Simulation(p)
    sim.init_state()
    sim.collect_enable(probes=probes, envelope_row=2, envelope_len=env_len, capacity=256,
                       envelope_halfwidth=0.5)
    st = sim.run(nsteps)
    got = sim.collect_read()
    orc = OracleSim(p, np.float32, math="fvm")
    orc.init_state()
    eta = np.float32(np.float32(p.nx) / np.float32(p.xmax))
    T_s, cfl_s, pr_s = [], [], []
    env = np.zeros(env_len, np.float32)
    for _ in range(nsteps):
        o = orc.run(1)
        T = np.float32(o["T"])
        if T <= 0:
            continue
        u1 = orc.get_state()[0]
        mdx, mdy = o["mdx"], o["mdy"]
        T_s.append(T)
        cfl_s.append(np.float32(orc.last_cfl()))
        row = []
        for (pi, pj) in probes:
            i, j = pi - mdx, pj - mdy
            row.append(u1[j, i] if 0 <= i < p.nx and 0 <= j < p.ny else np.float32(0))
        pr_s.append(row)
        j = 2 - mdy
        if 0 <= j < p.ny:
            for i in range(p.nx):
                lab = i + mdx
                if lab < env_len and abs(np.float32(np.float32(lab) / eta) - T) <= 0.5:
                    env[lab] = u1[j, i] if u1[j, i] > env[lab] else env[lab]
    assert st["mdx"] > 0 and got["steps"] == len(T_s) > 0
    np.testing.assert_array_equal(got["T"], np.array(T_s, np.float32))
    np.testing.assert_array_equal(got["cfl"], np.array(cfl_s, np.float32))
    np.testing.assert_array_equal(got["probes"], np.array(pr_s, np.float32))
    np.testing.assert_array_equal(got["envelope"], env)
    assert got["envelope"].max() > 0
    # the series empties on read; the envelope keeps accumulating
    sim.run(5)
    again = sim.collect_read()
    assert again["steps"] == 5 and np.all(again["envelope"] >= got["envelope"])
    sim.close()


def test_collection_overflow_stops_the_run():
    p = small_params(2, 64, 32)
    sim = Simulation(p)
    sim.init_state()
    sim.collect_enable(probes=[(10, 10)], capacity=4)
    with pytest.raises(_abi.FvError) as e:
        sim.run(10)
    assert e.value.status == _abi.FV_COLLECT_OVERFLOW
    assert sim.collect_read()["steps"] == 4
    sim.close()


def test_recorder_writes_the_frame_files(tmp_path):
    from fivonagi_gb300.export import Recorder

    p = small_params(0, 96, 48)
    sim = Simulation(p)
    sim.init_state()
    rec = Recorder(sim, str(tmp_path), dtprint=1.0)
    for _ in range(4):
        rec.frame_step()
    names = sorted(f.name for f in tmp_path.iterdir())
    for want in ("u1-0003.dat", "u1-cut-0003.dat", "u1max.dat", "microphone_4.dat", "u1-cfl.dat"):
        assert want in names
    assert rec.n_done > 0
    sim.close()


def test_pipelined_attempts_collect_like_a_run():
    """The pipelined calls (fv_steps_async / fv_step_wait) run the attempts
    in graphs of their own, with the collection launch after each one: with
    the window moving, the state, every attempt's T and the collected
    series equal those of one fv_run of the same steps."""
    p = small_params(0, 96, 48).replace(moving_domain=1, mdt=0.5, mdvx=1.0, mdvy=0.0)
    probes = [(20, 2), (40, 2), (55, 10)]
    nsteps = 70
    runs = []
    for pipelined in (False, True):
        sim = Simulation(p)
        sim.init_state()
        sim.collect_enable(probes=probes, envelope_row=2, envelope_len=4 * p.nx, capacity=256,
                           envelope_halfwidth=0.5)
        if pipelined:
            acc = 0
            while acc < nsteps:  # as many attempts as steps remain (a rejection needs another round)
                for st in sim.steps_pipelined(nsteps - acc):
                    acc += st["accepted"]
                    T = st["T"]
            assert acc == nsteps
        else:
            T = sim.run(nsteps)["T"]
        runs.append((sim.get_state(), sim.collect_read(), T, sim.stats()["mdx"]))
        sim.close()
    (a, ca, Ta, ma), (b, cb, Tb, mb) = runs
    assert ma == mb > 0 and np.float32(Ta) == np.float32(Tb)
    for f in range(3):
        np.testing.assert_array_equal(a[f], b[f])
    for key in ("T", "cfl", "probes", "envelope"):
        np.testing.assert_array_equal(ca[key], cb[key])
    assert ca["steps"] == cb["steps"] > 0
