"""Committed golden fixtures (tests/golden/, written by
tests/golden/make_golden.py from the oracle on seeded inputs): the oracle
must still reproduce them bit for bit, and the GPU library must match them
-- hits with the parity rule of the trace tests (kinds identical, ids
identical except near-edge hits or exact t ties, t within 1e-5 relative),
the small render within the render tests' tolerance, samples bit for bit."""
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
    assert rel < 0.02, rel
    g.close()
    z = _load("samplers.npz")
    for d in range(128):
        got = gpu.halton_samples(d, z["halton_indices"])
        assert np.array_equal(got.view(np.uint32), z["halton"][d].view(np.uint32)), d
