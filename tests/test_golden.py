"""Committed golden fixtures (tests/golden/, written by
tests/golden/make_golden.py from the oracle on seeded inputs): the oracle
must still reproduce them bit for bit, and the GPU library must match them
-- hits with the parity rule of the trace tests (kinds identical, ids
identical except near-edge hits or exact t ties, t within 1e-5 relative),
the small render within the render tests' bar (1e-6 relative RMSE), samples
bit for bit."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle.runner import OracleScene
from psychopath_gb300 import abi

from . import scene_cases as sc
from .golden import make_golden as mg

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _hits_fixture(name):
    z = _load("hits_%s.npz" % name)
    return z["rays"].view(abi.ray_dtype()), z["hits"].view(abi.hit_dtype())


@pytest.mark.parametrize("name", ["cornell", "sphere", "grid", "motion"])
def test_oracle_reproduces_hit_fixtures(oracle_lib, name):
    sd = {n: s for n, s, _ in mg.golden_ray_sets()}[name]
    rays, want = _hits_fixture(name)
    got, _, _, _ = OracleScene(sd).trace(rays, threads=2)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))


def test_oracle_reproduces_render_and_sampler_fixtures(oracle_lib):
    img, _ = OracleScene(mg.golden_render_scene()).render(threads=1)
    assert np.array_equal(img, _load("render_cornell16.npz")["xyz"])
    z = _load("samplers.npz")
    v = C.c_float()
    for d in range(128):
        for j, i in enumerate(z["halton_indices"]):
            assert oracle_lib.psyo_halton_sample(int(i), d, C.byref(v)) == 0
            assert np.float32(v.value) == z["halton"][d, j], (d, i)
    for si, s in enumerate(z["hash_seeds"]):
        for k, n in enumerate(z["hash_n"]):
            assert oracle_lib.psyo_hash_u32(int(n), int(s)) == z["hash_u32"][si, k]
            assert np.float32(oracle_lib.psyo_hash_u32_to_f32(int(n), int(s))) == z["hash_u32_to_f32"][si, k]
    for (i, scr), want in zip(z["golden_args"], z["golden"]):
        assert np.float32(oracle_lib.psyo_golden_ratio_sample(int(i), int(scr))) == want
    out = (C.c_float * 4)()
    for row, want in zip(z["sample_4d_args"], z["sample_4d"]):
        oracle_lib.psyo_get_sample_4d(*(int(v) for v in row), out)
        assert np.array_equal(np.array(list(out), dtype=np.float32), want), row
    for row, want in zip(z["wavelength_args"], z["wavelengths"]):
        oracle_lib.psyo_wavelengths(*(int(v) for v in row), out)
        assert np.array_equal(np.array(list(out), dtype=np.float32), want), row


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cornell", "sphere", "grid", "motion"])
def test_gpu_matches_hit_fixtures(gpu_lib, name):
    from psychopath_gb300 import gpu
    sd = {n: s for n, s, _ in mg.golden_ray_sets()}[name]
    rays, want = _hits_fixture(name)
    g = gpu.Scene(sd)
    tr = gpu.Tracer(g)
    for mode, minb in [(0, 4), (3, 10)]:  # the general and (when the scene allows) the static-scene traversal
        g.set_trace(mode, minb)
        got = tr.trace(rays)
        st = sc.compare_hits(got, want)
        assert st["kind_mismatch"] == 0 and st["unexplained"] == 0 and st["t_max_rel"] <= 1e-5, (mode, st)
    g.close()


@pytest.mark.gpu
def test_gpu_matches_render_and_sampler_fixtures(gpu_lib):
    from psychopath_gb300 import gpu
    g = gpu.Scene(mg.golden_render_scene())
    img, _ = gpu.Renderer(g).render()
    ref = _load("render_cornell16.npz")["xyz"].astype(np.float64)
    rel = np.sqrt(np.mean((img - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
    assert rel < 1e-6, rel  # measured 5.6e-8; the render tests' bar
    g.close()
    z = _load("samplers.npz")
    for d in range(128):
        got = gpu.halton_samples(d, z["halton_indices"])
        assert np.array_equal(got.view(np.uint32), z["halton"][d].view(np.uint32)), d


@pytest.mark.gpu
def test_gpu_samplers_bit_exact(gpu_lib):
    """The render path's samplers on the GPU equal the fixtures bit for bit:
    hash_u32, hash_u32_to_f32 (src/hash.rs:1-29), golden_ratio_sample
    (src/renderer.rs:728-737), get_sample_4d for the two Sobol-Burley sets and
    the hash sets (src/renderer.rs:698-725), and the camera's 4 hero
    wavelengths (src/renderer.rs:261-265, src/color.rs:20-43)."""
    from psychopath_gb300 import gpu
    z = _load("samplers.npz")
    n, seeds = z["hash_n"], z["hash_seeds"]
    args = np.zeros((len(seeds) * len(n), 5), dtype=np.uint32)
    args[:, 0] = np.tile(n, len(seeds))
    args[:, 1] = np.repeat(seeds, len(n))
    got = gpu.device_samplers("hash_u32", args)[:, 0].reshape(len(seeds), len(n))
    assert np.array_equal(got, z["hash_u32"])
    got = gpu.device_samplers("hash_u32_to_f32", args)[:, 0].reshape(len(seeds), len(n))
    assert np.array_equal(got, z["hash_u32_to_f32"].view(np.uint32))
    ga = z["golden_args"]
    args = np.zeros((len(ga), 5), dtype=np.uint32)
    args[:, :2] = ga
    assert np.array_equal(gpu.device_samplers("golden_ratio_sample", args)[:, 0], z["golden"].view(np.uint32))
    got = gpu.device_samplers("get_sample_4d", z["sample_4d_args"])
    assert np.array_equal(got, z["sample_4d"].view(np.uint32))
    wa = z["wavelength_args"]
    args = np.zeros((len(wa), 5), dtype=np.uint32)
    args[:, 0], args[:, 2], args[:, 3], args[:, 4] = wa[:, 0], wa[:, 1], wa[:, 2], wa[:, 3]
    assert np.array_equal(gpu.device_samplers("wavelengths", args), z["wavelengths"].view(np.uint32))
