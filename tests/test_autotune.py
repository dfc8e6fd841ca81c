"""The launch autotuner (fivonagi_gb300.autotune).

Every candidate -- CTA shape (warps per CTA x CTAs per SM x rows loaded
ahead), CTA count in waves and division -- gives the same bits, so the
tuner may pick any of them on speed alone; these tests check the candidate
set on CPU, and on the GPU that a tuned launch is cached, reused and still
the oracle's result.
"""
import numpy as np
import pytest

from fivonagi_gb300 import _abi, autotune


def test_candidates_cover_every_shape_and_both_divisions():
    c = list(autotune.candidates())
    assert sorted(s for s, d in c if d == _abi.FV_DIVISION_EXACT) == sorted(_abi.FV_CTA_SHAPES)
    assert (0, _abi.FV_DIVISION_FMA) in c
    assert len(set(c)) == len(c)


def test_cache_key_names_device_grid_and_variant():
    p = _abi.FvParams()
    p.nx, p.ny, p.exact = 512, 256, 1
    k = autotune._key(p, "GB300")
    assert k.startswith(f"v{autotune.CACHE_VERSION}|GB300|512x256|exact=1")


@pytest.mark.gpu
def test_tuned_launch_is_cached_and_matches_the_oracle(tmp_path, monkeypatch):
    from oracle.oracle import OracleSim
    from fivonagi_gb300 import Simulation
    from tests.helpers import perturbed, same_values, small_params

    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "autotune.json"))
    p = small_params(3, 300, 130)
    best = autotune.tune(p, steps=8)
    assert (best.shape, best.division) in set(autotune.candidates())
    assert autotune.tune(p) == best  # from the cache
    orc = OracleSim(p, np.float32, math="fvm")
    orc.init_state()
    u = perturbed(orc.get_state(), 5, 1e-4)
    orc.set_state(*u)
    so = orc.run(20)
    sim = Simulation(p)
    autotune.set_launch(sim, best)
    sim.set_state(*u)
    sg = sim.run(20)
    assert sg["rejected"] == so["rejected"]
    g, o = sim.get_state(), orc.get_state()
    assert all(same_values(g[f], o[f]) for f in range(3))
    sim.close()


def test_batch_cache_key_names_the_batch_shape():
    a = _abi.FvParams()
    a.nx, a.ny, a.exact = 256, 512, 1
    b = a.replace(nx=512)
    assert autotune._batch_key([a, b], "GB300") != autotune._batch_key([b, a], "GB300")
    assert autotune._batch_key([a, b], "GB300").startswith(f"v{autotune.CACHE_VERSION}|GB300|batch|2|")


@pytest.mark.gpu
def test_tuned_batch_launch_gives_the_same_bits(tmp_path, monkeypatch):
    from fivonagi_gb300 import Batch
    from tests.helpers import small_params

    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "autotune.json"))
    plist = [small_params(3, 300, 130), small_params(0, 96, 48), small_params(2, 200, 64)]
    blocks = autotune.tune_batch(plist, steps=4)
    assert autotune.tune_batch(plist) == blocks  # from the cache
    states = []
    for nb in (0, blocks):
        b = Batch(plist)
        b.set_launch(nb)
        b.init_state()
        b.run(15)
        states.append([b.get_state(k) for k in range(len(plist))])
        b.close()
    for k in range(len(plist)):
        for f in range(3):
            np.testing.assert_array_equal(states[0][k][f], states[1][k][f])
