"""fv_render: the headless display against its numpy restatement."""
import numpy as np
import pytest

from fivonagi_gb300 import Simulation, export
from tests.helpers import small_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("zoom,jcut", [(1, -1), (2, 10)])
def test_render_matches_numpy(zoom, jcut, tmp_path):
    p = small_params(3, 96, 64)
    sim = Simulation(p)
    sim.init_state()
    sim.run(80)
    u1 = sim.get_state()[0]
    w, h = p.nx // zoom, p.ny // zoom
    img = sim.render(zoom=zoom, jcut=jcut, plot_scale=0.5)
    ref = export.render_reference(u1, p.ampl, 0.5, w, h, zoom=zoom, jcut=jcut)
    assert img.shape == ref.shape
    diff = np.abs(img.astype(int) - ref.astype(int))
    assert diff.max() <= 1 and (diff == 0).mean() > 0.99
    assert len(np.unique(img[..., 0])) > 10  # a picture, not a flat colour
    export.write_png(str(tmp_path / "u1.png"), img)
    assert (tmp_path / "u1.png").stat().st_size > 100
    sim.close()
