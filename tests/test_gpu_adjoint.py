"""The discrete adjoint of the phased array's windowed loss.

The forward the adjoint records is the library's ordinary step, so its final
state equals fv_run's bit for bit. The gradient is checked against central
differences of the FP64 oracle run on the forward's recorded dt schedule
(the adjoint holds that schedule fixed).
"""
import numpy as np
import pytest

from fivonagi_gb300 import Simulation
from fivonagi_gb300.adjoint import Adjoint, array_loss_function, loss_window
from oracle.oracle import OracleSim
from tests.helpers import array_weights, same_values, small_params

pytestmark = pytest.mark.gpu

NX, NY, NSTEPS = 64, 48, 120
WIN = (14, 18, 8, 8, 60, NSTEPS)  # i0, j0, ni, nj, first, last


def _params():
    return small_params(4, NX, NY)


def _oracle_loss(p, amp, ph, dts, Ts):
    """The loss of the FP64 oracle on a fixed dt schedule."""
    q = p.replace(cflmax=1e30)
    o = OracleSim(q, np.float64)
    o.set_weights(np.asarray(amp, np.float64), np.asarray(ph, np.float64))
    o.init_state()
    i0, j0, ni, nj, first, last = WIN
    acc = 0.0
    for n in range(NSTEPS):
        o.set_scalars(dts[n], Ts[n], n)
        st = o.run(1)
        assert st["rc"] == 0 and st["accepted"] == 1
        if first <= n + 1 <= last:
            u1 = o.get_state()[0]
            acc += float(np.sum(u1[j0:j0 + nj, i0:i0 + ni] ** 2))
    return acc / ((last - first + 1) * ni * nj)


def test_adjoint_forward_is_the_plain_step_and_replay_reproduces_it():
    p = _params()
    amp, ph = array_weights(p.array_elems, 11, p.ampl)
    adj = Adjoint(p, loss_window(*WIN), NSTEPS, checkpoint_every=16)
    loss = adj.forward(amp, ph)
    sim = Simulation(p)
    sim.set_array_weights(amp, ph)
    sim.init_state()
    sim.run(NSTEPS)
    g, r = adj.get_state(), sim.get_state()
    for f in range(3):
        assert same_values(g[f], r[f])
    dts, Ts = adj.schedule()
    assert np.all(dts > 0) and np.all(np.diff(Ts) > 0)
    assert adj.replay(amp, ph) == loss
    assert loss > 0
    sim.close()
    adj.close()


def test_adjoint_gradient_matches_fp64_central_differences():
    p = _params()
    amp, ph = array_weights(p.array_elems, 11, p.ampl)
    adj = Adjoint(p, loss_window(*WIN), NSTEPS, checkpoint_every=16)
    loss = adj.forward(amp, ph)
    ga, gp = adj.backward()
    dts, Ts = adj.schedule()
    adj.close()
    # the FP64 oracle's loss on the same schedule is the FP32 loss to a few ulps
    l64 = _oracle_loss(p, amp, ph, dts, Ts)
    assert abs(l64 - loss) <= 1e-4 * loss
    g64 = []
    for k in (0, 3, 5, 7):
        for which in ("amp", "phase"):
            a = amp.astype(np.float64).copy()
            f = ph.astype(np.float64).copy()
            v = a if which == "amp" else f
            h = 1e-4 * (abs(v[k]) if which == "amp" else 1.0)
            v[k] += h
            lp = _oracle_loss(p, a, f, dts, Ts)
            v[k] -= 2 * h
            lm = _oracle_loss(p, a, f, dts, Ts)
            fd = (lp - lm) / (2 * h)
            got = ga[k] if which == "amp" else gp[k]
            g64.append((which, k, got, fd))
    scale = max(abs(fd) for *_, fd in g64)
    assert scale > 0
    for which, k, got, fd in g64:
        assert abs(got - fd) <= 2e-3 * scale, (which, k, got, fd)


def test_adjoint_gradient_matches_the_tangent_linear_model_per_component():
    """Every one of the 16 weights against the oracle's tangent-linear model
    along the same FP32 trajectory (the dual-number restatement), each
    within 1e-3 of its own value, and the FP64 tangent-linear model against
    FP64 central differences."""
    from oracle.oracle import schedule_loss, tlm_loss

    p = _params()
    amp, ph = array_weights(p.array_elems, 11, p.ampl)
    adj = Adjoint(p, loss_window(*WIN), NSTEPS, checkpoint_every=16)
    loss = adj.forward(amp, ph)
    ga, gp = adj.backward()
    dts, Ts = adj.schedule()
    adj.close()
    nelem = p.array_elems
    dirs = list(range(2 * nelem))
    l32, t32 = tlm_loss(p, amp, ph, dirs, dts, Ts, WIN, np.float32)
    assert abs(l32 - loss) <= 1e-9 * loss
    g = np.concatenate([ga, gp])
    rel = np.abs(g - t32) / np.abs(t32)
    print("small adjoint vs TLM32, per weight:", np.array2string(rel, precision=2))
    assert np.all(rel <= 1e-3), rel
    _, t64 = tlm_loss(p, amp, ph, dirs[:4] + dirs[nelem:nelem + 4], dts, Ts, WIN, np.float64)
    for r, k in enumerate(dirs[:4] + dirs[nelem:nelem + 4]):
        a = amp.astype(np.float64).copy()
        f = ph.astype(np.float64).copy()
        v, kk = (a, k) if k < nelem else (f, k - nelem)
        h = 1e-4 * (abs(v[kk]) if k < nelem else max(abs(v[kk]), 1.0))
        v[kk] += h
        lp = schedule_loss(p, a, f, dts, Ts, WIN)
        v[kk] -= 2 * h
        lm = schedule_loss(p, a, f, dts, Ts, WIN)
        fd = (lp - lm) / (2 * h)
        assert abs(t64[r] - fd) <= 1e-3 * abs(fd), (k, t64[r], fd)


def test_torch_function_returns_the_adjoint_gradients():
    torch = pytest.importorskip("torch")
    p = _params()
    amp, ph = array_weights(p.array_elems, 4, p.ampl)
    adj = Adjoint(p, loss_window(*WIN), NSTEPS)
    fn = array_loss_function()
    ta = torch.tensor(amp, dtype=torch.float32, requires_grad=True)
    tp = torch.tensor(ph, dtype=torch.float32, requires_grad=True)
    loss = fn.apply(ta, tp, adj)
    (3.0 * loss).backward()
    ga, gp = adj.backward()
    np.testing.assert_allclose(ta.grad.numpy(), np.float32(3.0 * ga), rtol=1e-6)
    np.testing.assert_allclose(tp.grad.numpy(), np.float32(3.0 * gp), rtol=1e-6)
    adj.close()


def test_replays_repeat_and_backward_needs_a_new_forward():
    p = _params()
    amp, ph = array_weights(p.array_elems, 2, p.ampl)
    adj = Adjoint(p, loss_window(*WIN), NSTEPS)
    adj.forward(amp, ph)
    l1 = adj.replay(amp * 1.01, ph)
    l2 = adj.replay(amp * 1.01, ph)
    assert l1 == l2
    with pytest.raises(Exception):
        adj.backward()
    adj.forward(amp, ph)
    adj.backward()
    adj.close()


def test_backward_repeats_and_keeps_the_final_state():
    """An odd step count leaves the final state in the second buffer; the
    backward's segment replays must not lose track of it."""
    p = _params()
    amp, ph = array_weights(p.array_elems, 5, p.ampl)
    n = NSTEPS - 1
    adj = Adjoint(p, loss_window(14, 18, 8, 8, 60, n), n, checkpoint_every=10)
    adj.forward(amp, ph)
    before = adj.get_state()
    ga1, gp1 = adj.backward()
    after = adj.get_state()
    ga2, gp2 = adj.backward()
    for f in range(3):
        assert same_values(before[f], after[f])
    assert np.array_equal(ga1, ga2) and np.array_equal(gp1, gp2)
    adj.close()



def test_batched_adjoint_equals_each_design_alone():
    """Three designs (own weights, own loss windows) through one
    fv_adjoint_batch: every loss, schedule and gradient equals the
    single-design adjoint's for that design, bit for bit, on two backward
    passes."""
    from fivonagi_gb300.adjoint import AdjointBatch

    p = _params()
    wins = [loss_window(14, 18, 8, 8, 60, NSTEPS), loss_window(30, 10, 6, 10, 40, NSTEPS - 10),
            loss_window(40, 30, 10, 6, 90, NSTEPS)]
    weights = [array_weights(p.array_elems, 20 + d, p.ampl) for d in range(3)]
    amp = np.stack([w[0] for w in weights])
    ph = np.stack([w[1] for w in weights])
    ab = AdjointBatch(p, wins, NSTEPS, checkpoint_every=16)
    losses = ab.forward(amp, ph)
    ga, gp = ab.backward()
    ga2, gp2 = ab.backward()
    assert np.array_equal(ga, ga2) and np.array_equal(gp, gp2)
    for d in range(3):
        adj = Adjoint(p, wins[d], NSTEPS, checkpoint_every=16)
        loss = adj.forward(amp[d], ph[d])
        g1, g2 = adj.backward()
        dts, Ts = adj.schedule()
        bdts, bTs = ab.schedule(d)
        adj.close()
        assert loss == losses[d]
        assert np.array_equal(dts, bdts) and np.array_equal(Ts, bTs)
        assert np.array_equal(g1, ga[d]) and np.array_equal(g2, gp[d]), d
    ab.close()
