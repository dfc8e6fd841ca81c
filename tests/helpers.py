"""Small-case parameter blocks and comparison helpers for the tests."""
import numpy as np

from fivonagi_gb300 import FvParams


def small_params(app: int, nx: int, ny: int, exact: int = 1) -> FvParams:
    """A small grid of each app, with amplitudes large enough to exercise
    the nonlinear terms and the limiter, and the source active at T0."""
    p = FvParams()
    p.app = app
    p.nx, p.ny = nx, ny
    p.cfl_even_only = 1
    p.exact = exact
    p.max_retries = 64
    p.cflmax, p.cflwhish, p.dtini = 1.0, 0.9, 0.005
    if app == 0:  # hifu-beam hooks, source active from T = -2
        p.xmax, p.ymax = (nx - 1) / 16, (ny - 1) / 16
        p.beta, p.diffdelta = 4.8, 2.974e-4
        p.ampl, p.frec, p.isp_a, p.isp_f, p.tide = 0.01, 1.0, 1.0, 40.0, 2.0
        p.mdvx, p.mdvy, p.mdt = 1.0, 0.0, 1e9
    elif app == 1:  # taylor-angle-xy hooks at pi/8
        p.xmax, p.ymax = 12.5, 12.5
        p.beta, p.diffdelta = 1.0, 1e-3
        p.isp_rhoa = float(np.float32(-1e-3))
        p.isp_c = 2.1972245773362196
        p.angle = float(np.float32(np.float32(3.1415926) / 8))
        p.mdt, p.tide, p.mdvx, p.mdvy = 6.25, 4.0, 1.0, 0.0
    elif app == 2:  # plane wave
        p.xmax, p.ymax = (nx - 1) / 16, (ny - 1) / 16
        p.beta, p.diffdelta = 3.5, 1e-4
        p.ampl, p.frec, p.angle, p.tide = 1e-2, 1.0, np.pi / 6, 0.0
    elif app == 3:  # focused beam
        p.xmax, p.ymax = (nx - 1) / 16, (ny - 1) / 16
        p.beta, p.diffdelta = 3.5, 5e-5
        p.ampl, p.frec, p.isp_f = 5e-2, 1.0, 60.0
        p.aperture, p.center, p.ramp_periods, p.tide = ny / 2, ny / 2, 1.0, 0.0
    else:  # phased array: 8 elements over about half the left edge
        p.xmax, p.ymax = (nx - 1) / 16, (ny - 1) / 16
        p.beta, p.diffdelta = 3.5, 5e-5
        p.ampl, p.frec = 5e-2, 1.0
        p.array_elems = 8
        p.aperture = 8 * max(1, (ny // 2) // 8)
        p.center, p.ramp_periods, p.tide = ny / 2, 1.0, 0.0
    return p


def array_weights(nelem: int, seed: int, ampl: float):
    """Element amplitudes ~ U[0.5, 1.5] * ampl and phases ~ U[0, 2 pi), FP32."""
    rng = np.random.default_rng(seed)
    amp = (rng.uniform(0.5, 1.5, nelem) * ampl).astype(np.float32)
    ph = rng.uniform(0.0, 2 * np.pi, nelem).astype(np.float32)
    return amp, ph


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.sqrt(np.sum(b * b))
    num = np.sqrt(np.sum((a - b) ** 2))
    return float(num / den) if den > 0 else float(num)


def same_values(a, b) -> bool:
    """Equal as numbers (+0 == -0), NaNs in the same places."""
    a = np.asarray(a)
    b = np.asarray(b)
    return bool(np.array_equal(a, b, equal_nan=True))


def perturbed(u, seed: int, scale: float):
    """A seeded perturbation of a state, to leave symmetric initial data."""
    rng = np.random.default_rng(seed)
    return [x + np.float32(scale) * rng.standard_normal(x.shape).astype(np.float32) for x in u]
