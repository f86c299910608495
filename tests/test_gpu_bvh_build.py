"""GPU-built mesh BVHs (PSY_BVH_GPU: Morton codes, radix sort, binary radix
tree, BVH4 collapse on the device).  The tree differs from the reference's
SAH tree, so hits are compared with the SAH-built scene under the bar of
the oracle parity tests: same hit kinds, same primitive except near-edge
hits or exact t ties, t within 1e-5 relative."""
import numpy as np
import pytest

from psychopath_gb300 import abi, gpu, scenes

from . import scene_cases as sc

pytestmark = pytest.mark.gpu


def _hits(sd, rays, **kw):
    g = gpu.Scene(sd, **kw)
    h = gpu.Tracer(g).trace(rays)
    return g, h


@pytest.mark.parametrize("case", ["grid", "sphere", "motion", "cornell"])
def test_gpu_bvh_hits_match_sah(gpu_lib, case):
    if case == "grid":
        sd, P, F = sc.grid_small(256, 128)
        rays = np.concatenate([scenes.incoherent_rays(P, F, 30000, seed=3), scenes.coherent_rays(120)])
    elif case == "sphere":
        sd = sc.sphere_small(32, 18, 4, 6, level=5)
        rays = sc.targeted_rays(30000, [-1, -1, -1], [1, 1, 1], [-3, -3, 3], [3, 3, 5], seed=2)
    elif case == "motion":
        sd = sc.motion_small()
        rays = sc.targeted_rays(30000, [-50, -50, -50], [50, 50, 50], [-60, -60, 60], [60, 60, 95], seed=4,
                                time_random=True)
    else:
        sd = sc.cornell()
        rays = sc.random_rays(30000, [-1.0, 0.0, -1.0], [1.0, 2.0, 1.0], seed=5, occl_frac=0.3, max_t=1.5)
    g0, ref = _hits(sd, rays)
    g1, got = _hits(sd, rays, bvh="gpu")
    st = sc.compare_hits(got, ref)
    assert st["kind_mismatch"] == 0, st
    assert st["unexplained"] == 0, st
    assert st["t_max_rel"] <= 1e-5, st
    # every mesh's tree order is a permutation of its triangles
    for oi, o in enumerate(sd.objects):
        if o["kind"] == abi.PSY_OBJ_MESH:
            order, nodes = g1.mesh_bvh_info(oi)
            assert sorted(order.tolist()) == list(range(o["indices"].shape[0]))
    assert g1.info()["max_stack"] >= 1
    g0.close()
    g1.close()


def test_gpu_bvh_fp16_conservative_and_render(gpu_lib):
    """FP16 child bounds encode the GPU-built tree conservatively (identical
    hits), and the rendered image matches the SAH-built scene's."""
    sd = sc.sphere_small(32, 18, 4, 6, level=5)
    rays = sc.targeted_rays(20000, [-1, -1, -1], [1, 1, 1], [-3, -3, 3], [3, 3, 5], seed=8)
    g1, a = _hits(sd, rays, bvh="gpu")
    g2, b = _hits(sd, rays, bvh="gpu", bounds="fp16")
    assert np.array_equal(a, b)
    img_gpu, _ = gpu.Renderer(g1).render()
    g0 = gpu.Scene(sd)
    img_sah, _ = gpu.Renderer(g0).render()
    d = np.sqrt(np.mean((img_gpu.astype(np.float64) - img_sah) ** 2)) / np.sqrt(np.mean(img_sah.astype(np.float64) ** 2))
    assert d < 0.005, d
    for g in (g0, g1, g2):
        g.close()


def test_gpu_bvh_small_meshes(gpu_lib):
    """Meshes of one to five triangles (a root leaf, a single node)."""
    for nt in (1, 2, 3, 4, 5):
        sd = scenes.SceneData(8, 8, 1)
        sh = sd.add_shader(abi.PSY_SHADER_LAMBERT)
        v = np.array([[i, 0, 0] for i in range(nt + 2)] + [[i, 1, 0] for i in range(nt + 2)], dtype=np.float32)
        idx = np.array([[i, i + 1, nt + 2 + i] for i in range(nt)], dtype=np.uint32)
        o = sd.add_mesh(v, idx)
        sd.add_instance(o, sh)
        sd.set_camera([scenes.look_at((0.5, 0.5, -3.0), (0.5, 0.5, 0.0))], [40.0])
        rays = sc.targeted_rays(2000, [0, 0, 0], [nt + 1, 1, 0], [-1, -1, -3], [nt + 2, 2, -2], seed=nt)
        g0, ref = _hits(sd, rays)
        g1, got = _hits(sd, rays, bvh="gpu")
        st = sc.compare_hits(got, ref)
        assert st["kind_mismatch"] == 0 and st["unexplained"] == 0, st
        g0.close()
        g1.close()
