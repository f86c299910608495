"""A scene read from .psy text renders on the GPU path as the oracle renders
the same parsed scene (the render parity bars of test_gpu_render.py), with
every object, light and shader kind of the file format in it."""
import numpy as np
import pytest

from oracle.runner import OracleScene
from psychopath_gb300 import gpu, psy_file

from .test_psy_file import SCENE

pytestmark = pytest.mark.gpu


def _rel_rmse(a, b):
    return float(np.sqrt(np.mean((a.astype(np.float64) - b) ** 2)) / max(1e-12, np.sqrt(np.mean(b.astype(np.float64) ** 2))))


@pytest.mark.parametrize("bounces", [2, 4])
def test_psy_scene_render_matches_oracle(gpu_lib, bounces):
    sd = psy_file.load_psy(SCENE, max_bounces=bounces).data
    g = gpu.Scene(sd)
    img, st = gpu.Renderer(g).render()
    ref, ost = OracleScene(sd).render(threads=8)
    assert np.isfinite(img).all() and img.max() > 0
    # measured 2.9e-8 relative image RMSE; the render tests' bar
    assert _rel_rmse(img, ref) < 1e-6, _rel_rmse(img, ref)
    assert abs(st["ray_count"] - ost["ray_count"]) <= 0.01 * ost["ray_count"]
    g.close()
