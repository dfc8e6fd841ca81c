"""Workload presets (no GPU needed)."""
from fivonagi_gb300 import configs


def test_config3_generator_is_seeded_and_in_range():
    a = configs.batched(64, seed=7)
    c = configs.batched(64, seed=7)
    assert [p.as_dict() for p in a] == [p.as_dict() for p in c]
    for p in a:
        assert p.nx in configs.SIDES and p.ny in configs.SIDES
        assert 1.0 <= p.beta <= 10.0 and 1e-6 <= p.diffdelta <= 1e-3 and 1e-4 <= p.ampl <= 1e-2
        cells = (p.nx - 1) / p.xmax
        assert 8 <= round(cells) <= 32
