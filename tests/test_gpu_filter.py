"""fv_filter_u1: the spectral low-pass against numpy's FFT."""
import numpy as np
import pytest

from fivonagi_gb300 import Simulation
from tests.helpers import rel_l2, small_params

pytestmark = pytest.mark.gpu


def _numpy_lowpass(u1, radius):
    ny, nx = u1.shape
    spec = np.fft.rfft2(u1.astype(np.float64))
    ky = np.fft.fftfreq(ny) * ny
    kx = np.arange(nx // 2 + 1)
    keep = (kx[None, :] ** 2 + ky[:, None] ** 2) <= radius * radius
    return np.fft.irfft2(spec * keep, s=u1.shape)


@pytest.mark.parametrize("nx,ny", [(64, 48), (90, 50)])
def test_lowpass_matches_numpy_and_leaves_the_state(nx, ny):
    p = small_params(2, nx, ny)
    sim = Simulation(p)
    rng = np.random.default_rng(3)
    u = [rng.standard_normal((ny, nx)).astype(np.float32) * np.float32(1e-3) for _ in range(3)]
    sim.set_state(*u)
    full = sim.filter_u1(radius=1e6)
    assert rel_l2(full, u[0]) < 1e-6
    for radius in (3.5, 12.0):
        got = sim.filter_u1(radius)
        ref = _numpy_lowpass(u[0], radius)
        assert rel_l2(got, ref) < 1e-5, radius
    dc = sim.filter_u1(0.0)  # only the mean survives
    assert np.allclose(dc, u[0].astype(np.float64).mean(), rtol=0, atol=1e-9)
    after = sim.get_state()
    for f in range(3):
        assert np.array_equal(after[f], u[f])
    sim.close()
