"""psy_autotune: the tuner times a probe render under candidate launch
configurations (trace kernel form and register budget, stack depth, queue
tile, sort-key width, wave size, CUDA graphs) and keeps the fastest.  Every
candidate must render the same image bit for bit, so the image after tuning
equals the image before."""
import numpy as np
import pytest

from psychopath_gb300 import gpu

from . import scene_cases as sc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["sphere", "motion"])
def test_autotune_keeps_image(gpu_lib, case):
    s = sc.sphere_small(48, 27, 8, 6, level=4) if case == "sphere" else sc.motion_small(48, 27, 8, 2)
    g = gpu.Scene(s)
    r = gpu.Renderer(g)
    before, _ = r.render()
    res = g.autotune(probe_paths=4096, repeats=1)
    # mode 3 (the static-scene traversal) is a candidate only on static scenes
    assert res["trace_mode"] in ((0, 1, 3) if g.flags()["static_fast"] else (0, 1))
    budgets = {0: (4, 5, 6, 8), 1: (4, 6, 8), 3: (8, 10, 12)}
    assert res["minb"] in budgets[res["trace_mode"]]
    assert res["stack"] >= g.info()["max_stack"]
    assert res["sort_bits"] in (0, 4, 10, 13, 16, 19, 25)
    assert res["shade_minb"] in (4, 6, 8)
    assert res["candidates"] >= 17
    assert 0 < res["best_s"] <= res["default_s"]
    after, _ = r.render()
    assert np.array_equal(before, after)
    # the device path with the chosen configuration (graphs included) agrees too
    torch = pytest.importorskip("torch")
    d = torch.zeros(before.size, dtype=torch.float32, device="cuda")
    r.render_device(d.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy().reshape(before.shape), before)
    g.close()


def test_autotune_wave_size_bounded_and_image_unchanged(gpu_lib):
    """An image larger than the probe band gets the larger-wave step; a
    caller's max_wave_mib bounds it, and the image is the same bit for bit
    whatever wave size is chosen (paths are independent)."""
    s = sc.sphere_small(1024, 1024, 24, 2, level=3)  # 25.2M paths: more than the 16M probe band
    g = gpu.Scene(s, shading="f32")
    r = gpu.Renderer(g)
    g.set_launch(0, 1 << 22)
    before, _ = r.render()
    res = g.autotune(repeats=1, max_wave_mib=64)  # no larger wave fits in 64 MiB
    assert res["wave_paths"] <= 1 << 24
    res2 = g.autotune(repeats=1)
    assert res2["wave_paths"] <= 1024 * 1024 * 24
    after, _ = r.render()
    assert np.array_equal(before, after)
    g.close()
