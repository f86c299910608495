"""Renderer parity: GPU renders (camera -> wavefront light paths -> XYZ
accumulation) against the oracle's bucket renderer on the same scene and
seed.  Both evaluate the same sample sequences with the same f32/f64
operations, so images agree to rounding: they are not bit-identical because
sin/cos/acos/log come from different math libraries (CUDA vs the host libm,
1-2 ulp apart) and the difference grows along a path's bounces.

Bars (measured on a GB300 on these scenes, then a margin of about 7x):
relative image RMSE below RENDER_REL = 1e-6 (measured at most 1.4e-7) and
no more than RENDER_OFF = 0.1% of pixels beyond 1e-4 relative difference
(measured 0).  The f32 shading variant is held to its own measured error
with the same margin, inside its 1% precision budget."""
import numpy as np
import pytest

from oracle.runner import OracleScene
from psychopath_gb300 import gpu

from . import scene_cases as sc

pytestmark = pytest.mark.gpu


def rel_rmse(a, b):
    return float(np.sqrt(np.mean((a.astype(np.float64) - b) ** 2)) / max(1e-12, np.sqrt(np.mean(b.astype(np.float64) ** 2))))


def frac_off(a, b, tol=1e-4):
    d = np.abs(a.astype(np.float64) - b) / np.maximum(np.abs(b), 1e-3)
    return float(np.mean(d.max(axis=-1) > tol))


# Image bars of the renders against the oracle (relative image RMSE; share of
# pixels beyond 1e-4 relative difference).
RENDER_REL, RENDER_OFF = 1e-6, 0.001
# Per-path bars of test_paths_match_oracle_samples (measured: at most 1 of
# 2,048 paths beyond 1e-4 relative, the 4-bounce Cornell box).
PATH_REL, PATH_ABS, PATH_DIVERGED = 1e-4, 1e-7, 0.002


def _render_both(s):
    g = gpu.Scene(s)
    img, st = gpu.Renderer(g).render()
    o = OracleScene(s)
    ref, ost = o.render(threads=8)
    return img, ref, st, ost, g


@pytest.mark.parametrize("bounces", [2, 4])
def test_cornell_render(gpu_lib, bounces):
    s = sc.cornell(32, 32, 8, bounces)
    img, ref, st, ost, g = _render_both(s)
    assert np.isfinite(img).all()
    assert rel_rmse(img, ref) < RENDER_REL, rel_rmse(img, ref)
    assert frac_off(img, ref) <= RENDER_OFF, frac_off(img, ref)
    assert st["samples"] == 32 * 32 * 8
    # both count the same rays up to rare divergent paths
    assert abs(st["ray_count"] - ost["ray_count"]) <= 0.01 * ost["ray_count"]


def test_sphere_ggx_render(gpu_lib):
    s = sc.sphere_small(24, 16, 4, 6, level=3)
    img, ref, st, ost, g = _render_both(s)
    assert rel_rmse(img, ref) < RENDER_REL, rel_rmse(img, ref)
    assert frac_off(img, ref) <= RENDER_OFF, frac_off(img, ref)


def test_motion_render(gpu_lib):
    s = sc.motion_small(24, 16, 4, 2)
    img, ref, st, ost, g = _render_both(s)
    assert rel_rmse(img, ref) < RENDER_REL, rel_rmse(img, ref)
    assert frac_off(img, ref) <= RENDER_OFF, frac_off(img, ref)


def test_render_deterministic_and_bucket(gpu_lib):
    s = sc.cornell(32, 32, 4, 2)
    g = gpu.Scene(s)
    r = gpu.Renderer(g)
    a, _ = r.render()
    b, _ = r.render()
    assert np.array_equal(a, b)
    # a bucket renders the same pixels as the full image
    bk, _ = r.render_bucket(8, 4, 16, 12)
    assert np.array_equal(bk, a[4:16, 8:24])
    # small waves (many waves per image) give the same image
    g.set_launch(wave_paths=2048)
    c, _ = r.render()
    assert np.array_equal(a, c)
    # crop renders only the cropped pixels
    d, _ = r.render(crop=(4, 4, 9, 7))
    assert np.array_equal(d[4:8, 4:10], a[4:8, 4:10])
    assert not d[:4].any()


def test_interleaved_rows_equal_whole_image(gpu_lib):
    """psy_render_rows_device (one rank's share of a multi-GPU frame): rows
    first, first + step, ... equal the whole-image render's rows bit for bit,
    with small waves too (several waves per share)."""
    import torch
    s = sc.sphere_small(24, 17, 4, 6, level=3)
    g = gpu.Scene(s)
    r = gpu.Renderer(g)
    full, _ = r.render()
    for wave in (0, 96):
        if wave:
            g.set_launch(wave_paths=wave * 4)
        for step in (1, 2, 3, 8):
            for first in range(min(step, 3)):
                n = len(range(first, s.height, step))
                d = torch.full((n * s.width * 3,), -1.0, dtype=torch.float32, device="cuda")
                st = r.render_rows_device(first, step, d.data_ptr(), stats=True)
                torch.cuda.synchronize()
                got = d.cpu().numpy().reshape(n, s.width, 3)
                assert np.array_equal(got, full[first::step]), (wave, step, first)
                assert st["samples"] == n * s.width * s.spp
    g.close()


def test_bucket_rejects_bad_arguments(gpu_lib):
    """A bucket whose x + w or y + h passes 2^32 (checked in 64 bits), an
    empty bucket and spp == 0 are rejected before any launch, by both bucket
    entry points."""
    import ctypes as C
    import torch
    from psychopath_gb300 import abi
    g = gpu.Scene(sc.cornell(32, 32, 4, 2))
    out = np.zeros(32 * 32 * 3, dtype=np.float32)
    d_out = torch.zeros(32 * 32 * 3, dtype=torch.float32, device="cuda")
    cases = [((0xFFFFFFF0, 0, 32, 8), 4), ((0, 0xFFFFFFF0, 8, 32), 4), ((0, 0, 0, 8), 4), ((0, 0, 8, 8), 0),
             ((30, 0, 4, 4), 4)]
    for (x, y, w, h), spp in cases:
        b = abi.PsyBucket(x, y, w, h)
        assert gpu_lib.psy_render_bucket(g.h, C.byref(b), spp, 0, out.ctypes.data, None) == abi.PSY_E_INVALID
        assert gpu_lib.psy_render_bucket_noalloc(g.h, C.byref(b), spp, 0, C.c_void_p(d_out.data_ptr()),
                                                 None) == abi.PSY_E_INVALID
    g.close()


@pytest.mark.parametrize("case", ["cornell", "ggx", "motion"])
def test_paths_match_oracle_samples(gpu_lib, case):
    """Per-sample results of one bucket, GPU vs oracle, path by path: the
    hero wavelength of every sample bit for bit, and each path's final
    4-wavelength colour within PATH_REL relative (PATH_ABS absolute for
    near-zero values) for all but PATH_DIVERGED of the paths (a path whose
    direction flips after a last-ulp sin/cos difference)."""
    s = {"cornell": sc.cornell(32, 32, 16, 4), "ggx": sc.sphere_small(32, 18, 16, 6, level=3),
         "motion": sc.motion_small(32, 18, 16, 2)}[case]
    x, y, w, h = 8, 4, 16, 8
    o = OracleScene(s)
    col, wl, _ = o.render_paths(x, y, w, h)
    g = gpu.Scene(s)
    gcol, gwl = gpu.Renderer(g).render_paths(x, y, w, h)
    assert np.array_equal(gwl.view(np.uint32), wl.view(np.uint32))
    fin = np.isfinite(col).all(axis=1) & np.isfinite(gcol).all(axis=1)
    assert np.array_equal(np.isfinite(col).all(axis=1), np.isfinite(gcol).all(axis=1))
    d = np.abs(gcol[fin].astype(np.float64) - col[fin])
    bad = (d > PATH_REL * np.abs(col[fin]) + PATH_ABS).any(axis=1)
    print("%s: %d paths, %d beyond %.0e, max abs diff %.3e" % (case, len(col), bad.sum(), PATH_REL, d.max()))
    assert bad.mean() <= PATH_DIVERGED, (bad.sum(), len(bad))
    g.close()


@pytest.mark.parametrize("bits", [4, 10, 13, 16, 19, 25, 31])
def test_ray_binning_does_not_change_image(gpu_lib, bits):
    """Binning the wavefront queue by ray key only reorders independent
    paths: the image is bit-identical to the unbinned one."""
    s = sc.sphere_small(24, 16, 4, 6, level=3)
    g = gpu.Scene(s)
    r = gpu.Renderer(g)
    g.set_sort(0)
    a, _ = r.render()
    g.set_sort(bits)
    b, _ = r.render()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("graph", [False, True])
def test_radix_queue_order_many_tiles(gpu_lib, graph):
    """Two-point radix ordering of the wavefront queues over many sort tiles
    (~98k paths, the queue length read on the device), launched kernel by
    kernel and replayed from a CUDA graph: bit-identical image."""
    import torch
    s = sc.sphere_small(128, 96, 8, 6, level=3)
    g = gpu.Scene(s)
    r = gpu.Renderer(g)
    g.set_sort(0)
    a, _ = r.render()
    g.set_graph(graph)
    d = torch.zeros(s.height * s.width * 3, dtype=torch.float32, device="cuda")
    for bits in (19, 25):
        g.set_sort(bits)
        r.render_device(d.data_ptr())  # no stats: the graph path when enabled
        torch.cuda.synchronize()
        assert np.array_equal(a, d.cpu().numpy().reshape(a.shape))


def test_f32_shading_precision_error(gpu_lib):
    """The f32 shading variant (no FP64 outside the triangle retest) against
    the oracle and the FP64 oracle: inside the 1% precision budget of the
    optimized form, and held to its measured error (1.1e-5 relative RMSE on
    this GGX scene) with a 10x margin."""
    s = sc.sphere_small(48, 27, 16, 6, level=4)
    g = gpu.Scene(s, shading="f32")
    img, _ = gpu.Renderer(g).render()
    ref, _ = OracleScene(s).render(threads=8)
    ref64, _ = OracleScene(s, f64=True).render(threads=8)
    assert rel_rmse(img, ref) < 1e-4, rel_rmse(img, ref)
    assert rel_rmse(img, ref64) < 1e-4, rel_rmse(img, ref64)


@pytest.mark.parametrize("minb", [6, 8])
def test_shade_register_budget_does_not_change_image(gpu_lib, minb):
    """The shading kernel compiled for more resident blocks (fewer registers)
    computes the same paths: bit-identical image, both precisions."""
    s = sc.sphere_small(24, 16, 4, 6, level=3)
    for shading in ("f64", "f32"):
        g = gpu.Scene(s, shading=shading)
        r = gpu.Renderer(g)
        a, _ = r.render()
        g.set_shade(minb)
        b, _ = r.render()
        assert np.array_equal(a, b)
        g.close()


@pytest.mark.parametrize("mode,minb", [(1, 8), (2, 4), (3, 8), (3, 12), (5, 10)])
def test_trace_mode_does_not_change_image(gpu_lib, mode, minb):
    """The wavefront renders the same image with the persistent, the
    warp-packet, the static-scene traversal and its lane-refill form (on the
    static scene; the motion scene falls back to the general kernel) as with
    one thread per ray."""
    for s in (sc.sphere_small(24, 16, 4, 6, level=3), sc.motion_small(24, 16, 4, 2)):
        g = gpu.Scene(s)
        r = gpu.Renderer(g)
        a, _ = r.render()
        g.set_trace(mode, minb)
        b, _ = r.render()
        assert np.array_equal(a, b)
        g.close()


@pytest.mark.parametrize("grid", [-1, 4, 152])
def test_wavefront_grid_does_not_change_image(gpu_lib, grid):
    """Wavefront kernels launched on each kernel's resident blocks (-1) or a
    small fixed grid (4 blocks: every thread strides over ~48 queue slots)
    instead of one thread per queue slot, with the general and the
    static-scene traversal and binned queues: bit-identical image."""
    s = sc.sphere_small(64, 48, 8, 6, level=3)
    for shading in ("f64", "f32"):
        g = gpu.Scene(s, shading=shading)
        r = gpu.Renderer(g)
        a, _ = r.render()
        for mode, minb, bits in ((0, 4, 0), (3, 10, 19)):
            g.set_trace(mode, minb)
            g.set_sort(bits)
            g.set_launch(grid=grid)
            b, _ = r.render()
            assert np.array_equal(a, b), (shading, mode, grid)
            g.set_launch(grid=0)
        g.close()


@pytest.mark.parametrize("tail", [1, 6, 15])
def test_resident_tail_does_not_change_image(gpu_lib, tail):
    """The last `tail` wavefront iterations on resident grids (15 = all of
    the scene's 2 * 6 + 3 iterations), the rest on grids sized by the wave,
    with the general and the static-scene traversal: bit-identical image."""
    s = sc.sphere_small(64, 48, 8, 6, level=3)
    g = gpu.Scene(s, shading="f32")
    r = gpu.Renderer(g)
    a, _ = r.render()
    for mode, minb, bits in ((0, 4, 0), (3, 10, 19)):
        g.set_trace(mode, minb)
        g.set_sort(bits)
        g.set_resident_tail(tail)
        b, _ = r.render()
        assert np.array_equal(a, b), (mode, tail)
        g.set_resident_tail(0)
    g.close()


@pytest.mark.parametrize("case", ["cornell", "mesh_stress", "light_tree_64"])
def test_color_spectrum_tables(gpu_lib, case):
    """The f32 form takes each constant XYZ colour's spectrum (shader
    colours, light and distant-light colours, the background) from a table
    of its combined Meng point spectra: at any hero wavelength the same
    value as the upsampling up to rounding (bar 1e-5 relative), and
    exactly 0 where the upsampling gives 0."""
    from psychopath_gb300 import scenes
    if case == "cornell":
        s = sc.cornell()
    elif case == "mesh_stress":
        s = scenes.mesh_stress(64, 36, 1, level=4)
    else:
        s = sc.motion_small(48, 27, 8, 2, lights=64)
    g = gpu.Scene(s, shading="f32")
    rng = np.random.default_rng(3)
    heros = np.concatenate([rng.uniform(380.0, 700.0, 4000), [380.0, 459.9999, 460.0, 699.9999]]).astype(np.float32)
    ex, tb = g.color_spectra(heros)
    g.close()
    assert ex.shape[0] >= 2 and ex.shape == tb.shape
    assert np.array_equal(ex == 0.0, tb == 0.0)
    scale = np.maximum(np.abs(ex), 1e-30)
    rel = np.abs(tb.astype(np.float64) - ex) / scale
    assert rel.max() < 1e-5, rel.max()


def test_f32_shading_sphere_lights(gpu_lib):
    """The f32 variant on a motion scene lit by sphere lights (cone sampling
    and its pdf in f32): within 1% relative RMSE of the oracle, and no
    non-finite pixel the oracle does not also have."""
    s = sc.motion_small(48, 27, 8, 2)
    g = gpu.Scene(s, shading="f32")
    img, _ = gpu.Renderer(g).render()
    ref, _ = OracleScene(s).render(threads=8)
    bad_g = ~np.isfinite(img).all(axis=-1)
    bad_o = ~np.isfinite(ref).all(axis=-1)
    assert not (bad_g & ~bad_o).any()
    ok = ~(bad_g | bad_o)
    # measured 1.1e-6: the f32 shading kernels round a product feeding a sum
    # once (FMA contraction), the oracle twice (2.2e-8 without contraction);
    # the sphere lights' cone sampling is f32 in both
    assert rel_rmse(img[ok], ref[ok]) < 1e-5, rel_rmse(img[ok], ref[ok])


def test_speculative_traversal_render(gpu_lib):
    """The speculative traversal's image equals the static-scene traversal's
    up to tie-broken hits (none expected on this scene at this size)."""
    s = sc.sphere_small(24, 16, 4, 6, level=3)
    g = gpu.Scene(s)
    r = gpu.Renderer(g)
    g.set_trace(3, 8)
    a, _ = r.render()
    g.set_trace(4, 8)
    b, _ = r.render()
    rel = np.sqrt(np.mean((a.astype(np.float64) - b) ** 2)) / np.sqrt(np.mean(a.astype(np.float64) ** 2))
    assert rel < 1e-3
    g.close()


def test_light_tree_64_lights(gpu_lib):
    """64 sphere lights (the motion + instancing configuration's count): the
    oracle's 8-ary light tree has inner levels below the root, so light
    selection descends LightTree::select (src/accel/light_tree.rs:135-201)
    more than one level; the GPU render matches the oracle's."""
    s = sc.motion_small(48, 27, 8, 2, lights=64)
    o = OracleScene(s)
    nodes, leaves, depth = o.light_tree_info()
    assert leaves == 64 and depth >= 3, (nodes, leaves, depth)
    img, ref, st, ost, g = _render_both(s)
    ok = np.isfinite(img).all(-1) & np.isfinite(ref).all(-1)
    print("64 lights: rel RMSE %.3e, pixels off %.4f" % (rel_rmse(img[ok], ref[ok]), frac_off(img[ok], ref[ok])))
    assert rel_rmse(img[ok], ref[ok]) < RENDER_REL, rel_rmse(img[ok], ref[ok])
    assert frac_off(img[ok], ref[ok]) < RENDER_OFF, frac_off(img[ok], ref[ok])


def test_thin_lens_camera_motion(gpu_lib):
    """Thin lens (aperture radii and focus distances keyed over time) on a
    moving camera with 3 transform keys and 2 field-of-view keys
    (Camera::generate_ray, src/camera.rs:74-102; square_to_circle,
    src/sampling/monte_carlo.rs:10-32): GPU render against the oracle."""
    s = sc.cornell_lens(32, 32, 8, 2)
    img, ref, st, ost, g = _render_both(s)
    assert np.isfinite(img).all()
    print("lens: rel RMSE %.3e, pixels off %.4f" % (rel_rmse(img, ref), frac_off(img, ref)))
    assert rel_rmse(img, ref) < RENDER_REL, rel_rmse(img, ref)
    assert frac_off(img, ref) < RENDER_OFF, frac_off(img, ref)
