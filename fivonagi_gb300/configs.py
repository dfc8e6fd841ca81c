"""Workload presets: the parameter blocks of the benchmark configurations.

Config 1: plane wave 512x512 (the app's defaults, fv_default_params).
Config 2: focused beam 4096x2048 (the app's defaults).
Config 3: a batch of focused-beam simulations of uneven sizes and physics,
          drawn from a base seed.
"""
from __future__ import annotations

import numpy as np

from . import _abi
from ._abi import FvParams

SIDES = (256, 512, 1024, 2048)


def config1() -> FvParams:
    return _abi.default_params(_abi.FV_APP_PLANE_WAVE)


def config2() -> FvParams:
    return _abi.default_params(_abi.FV_APP_FOCUSED_BEAM)


def batched(n: int = 64, seed: int = 0, sides=SIDES, exact: int = 1) -> list[FvParams]:
    """n focused-beam simulations: NX and NY drawn independently from
    `sides`; beta ~ U[1, 10]; dissipation ~ logU[1e-6, 1e-3]; source
    amplitude ~ logU[1e-4, 1e-2] (Mach); 8..32 cells per wavelength. The
    aperture is NY/2 centred on NY/2 and the focus is 0.75 NX cells."""
    rng = np.random.default_rng(seed)
    base = _abi.default_params(_abi.FV_APP_FOCUSED_BEAM)
    out = []
    for _ in range(n):
        nx = int(rng.choice(sides))
        ny = int(rng.choice(sides))
        cells = int(rng.integers(8, 33))
        beta = float(rng.uniform(1.0, 10.0))
        delta = float(10.0 ** rng.uniform(-6.0, -3.0))
        ampl = float(10.0 ** rng.uniform(-4.0, -2.0))
        out.append(base.replace(
            nx=nx, ny=ny, xmax=(nx - 1) / cells, ymax=(ny - 1) / cells, beta=beta, diffdelta=delta,
            ampl=ampl, aperture=ny / 2, center=ny / 2, isp_f=0.75 * nx, exact=exact))
    return out
