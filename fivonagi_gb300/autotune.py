"""Launch-shape autotuner for the step kernel.

The step kernel has two free launch parameters: the number of persistent
CTAs whose warps share the grid's (window, row) work (fv_set_launch), and
the division it computes with (fv_set_division: FMA division with a fix-up
pass, or exact division with no fix-up work; the results are the same bit
for bit). More waves keep every SM full to the end but repeat the streaming
loop's warm-up rows on shorter segments; exact division costs the step
kernel a few percent and saves the fix-up pass. The best pair depends on
the grid size. `tune` times each pair, in waves of the CTAs resident at
once, on a scratch copy of the simulation, and caches the winner per
(device, grid, variant) in a JSON file next to the library.
"""
from __future__ import annotations

import json
import os

from . import _abi
from ._abi import FvParams

CACHE = os.path.join(_abi.LIB_DIR, "autotune.json")
WAVES = (1, 2, 3, 4, 6, 8)


def _key(params: FvParams, device: str) -> str:
    return f"{device}|{params.nx}x{params.ny}|exact={params.exact}"


def _load() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def tune(params: FvParams, steps: int = 40, refresh: bool = False) -> tuple[int, int]:
    """Best (CTA count, division mode) for `params` on the current device
    (cached). Timing is the library's own (fv_time_run: CUDA events around
    ordinary launches on the handle's stream)."""
    from .solver import Simulation

    device = _abi.device_name()
    key = _key(params, device)
    cache = _load()
    if key in cache and not refresh and "division" in cache[key]:
        return int(cache[key]["blocks"]), int(cache[key]["division"])
    sim = Simulation(params)
    try:
        sim.init_state()
        sim.run(10)
        _, resident = sim.get_launch()
        results = {}
        for mode in (_abi.FV_DIVISION_FMA, _abi.FV_DIVISION_EXACT):
            sim.set_division(mode)
            for w in WAVES:
                b = w * resident
                try:
                    sim.set_launch(b)
                except _abi.FvError:
                    continue
                sim.run(4)
                results[(b, mode)] = sim.time_run(steps) / steps
                sim.sync()
        best = min(results, key=results.get)
    finally:
        sim.close()
    cache[key] = {"blocks": best[0], "division": best[1], "ms_per_step": results[best],
                  "candidates": {f"{b}/{'exact' if m else 'fma'}": v for (b, m), v in sorted(results.items())}}
    _store(cache)
    return best


def apply(sim, refresh: bool = False) -> tuple[int, int]:
    """Tune for `sim`'s parameters and set its launch shape and division;
    returns (CTAs, division mode)."""
    b, m = tune(sim.params, refresh=refresh)
    sim.set_launch(b)
    sim.set_division(m)
    return b, m
