"""Tracer::trace parity: the GPU closest-hit / any-hit results against the
oracle's packet traversal on the same rays, hit by hit.  Primitive and
instance ids must agree except at near-edge hits and exact t ties, and t must
agree to 1e-5 relative (it is bit-exact in practice: same arithmetic)."""
import numpy as np
import pytest

from oracle.runner import OracleScene
from psychopath_gb300 import abi, gpu, scenes

from . import scene_cases as sc

pytestmark = pytest.mark.gpu


def _run(scene_data, rays, bounds="fp32", full=False):
    g = gpu.Scene(scene_data, bounds=bounds)
    o = OracleScene(scene_data)
    tr = gpu.Tracer(g)
    if full:
        hg, fg = tr.trace(rays, full=True)
    else:
        hg, fg = tr.trace(rays), None
    ho, fo, _, _ = o.trace(rays, threads=8, full=full)
    assert tr.rays_traced() == len(rays)
    g.close()
    return hg, ho, fg, fo


def _assert_parity(st, min_surface=1):
    assert st["kind_mismatch"] == 0, st
    assert st["unexplained"] == 0, st
    assert st["surface"] >= min_surface, st
    assert st["t_max_rel"] <= 1e-5, st


def test_cornell_random_rays(gpu_lib):
    rays = sc.random_rays(20000, [-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], seed=1)
    hg, ho, _, _ = _run(sc.cornell(), rays)
    st = sc.compare_hits(hg, ho)
    _assert_parity(st, 15000)
    assert st["t_bit_exact"] == 1.0, st


def test_exact_edge_and_vertex_hits(gpu_lib):
    """Rays straight down through the vertices, edges and diagonals of a flat
    integer grid: every edge function the watertight test computes for the
    hit triangle is exactly zero somewhere, so the f64 retest
    (src/surface/triangle.rs:82-86) decides.  The GPU must pick the same
    triangle as the oracle at every such shared edge, with the same t and
    barycentrics, bit for bit, with FP32 and FP16 child bounds and the
    static-scene traversal.

    With FP16 bounds every oracle hit is found, at the same t.  The rays run
    exactly in faces of the flat grid's boxes (origin on the face, direction
    component 0): there the f32 slab distance is 0 * inf = NaN and the f32
    box test culls the box, while the outward-rounded FP16 box holds the ray
    strictly inside.  So FP16 visits more boxes: at a shared edge it can
    find another of the triangles tied at exactly that t first (an exact
    tie, allowed by the trace parity rule), and on the grid's border it finds
    edge hits the f32 boxes cull -- hits gained, never one lost."""
    s, rays = sc.flat_grid_edges(8)
    o = OracleScene(s)
    ho, _, _, _ = o.trace(rays, threads=1)
    bmin = np.minimum(np.minimum(ho["b0"], ho["b1"]), ho["b2"])
    hit = ho["kind"] == abi.PSY_HIT_SURFACE
    assert (bmin[hit] == 0).all() and hit.sum() >= 200
    for bounds, modes in (("fp32", [(0, 4), (3, 10)]), ("fp16", [(0, 4), (3, 10)])):
        g = gpu.Scene(s, bounds=bounds)
        tr = gpu.Tracer(g)
        for mode, minb in modes:
            g.set_trace(mode, minb)
            hg = tr.trace(rays)
            if bounds == "fp32":
                for f in ("kind", "prim", "inst", "t", "b0", "b1", "b2"):
                    assert np.array_equal(hg[f], ho[f]), (bounds, mode, f)
            else:
                assert np.array_equal(hg["kind"][hit], ho["kind"][hit]) and np.array_equal(hg["t"][hit], ho["t"][hit])
                other = hit & (hg["prim"] != ho["prim"])
                gmin = np.minimum(np.minimum(hg["b0"], hg["b1"]), hg["b2"])
                assert (gmin[other] == 0).all()  # the other triangle is hit on its edge too: a tie
                same = hit & ~other
                for f in ("b0", "b1", "b2"):
                    assert np.array_equal(hg[f][same], ho[f][same]), (bounds, mode, f)
                gained = ~hit & (hg["kind"] == abi.PSY_HIT_SURFACE)
                o = rays["orig"]
                border = (o[:, 0] == 0) | (o[:, 0] == 8) | (o[:, 2] == 0) | (o[:, 2] == 8)
                assert not (gained & ~border).any() and (hg["kind"][~hit & ~gained] == ho["kind"][~hit & ~gained]).all()
        g.close()


def test_cornell_occlusion_and_max_t(gpu_lib):
    rays = sc.random_rays(20000, [-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], seed=2, occl_frac=0.5, max_t=3.0)
    hg, ho, _, _ = _run(sc.cornell(), rays)
    st = sc.compare_hits(hg, ho)
    _assert_parity(st, 100)
    assert st["occluded"] > 1000


def test_displaced_sphere(gpu_lib):
    s = sc.sphere_small(level=5)
    rays = sc.targeted_rays(30000, [-1.1, -0.1, -1.1], [1.1, 2.1, 1.1], [-4, 0.05, -4], [4, 4, 4], seed=3)
    hg, ho, _, _ = _run(s, rays)
    st = sc.compare_hits(hg, ho)
    _assert_parity(st, 20000)
    assert st["prim_mismatch"] <= 5, st


def test_motion_instances(gpu_lib):
    s = sc.motion_small()
    rays = sc.targeted_rays(30000, [-50, -50, -50], [50, 50, 50], [-60, -60, 60], [60, 60, 95], seed=4,
                            time_random=True)
    hg, ho, _, _ = _run(s, rays)
    st = sc.compare_hits(hg, ho)
    _assert_parity(st, 200)


def test_grid_incoherent(gpu_lib):
    s, P, F = sc.grid_small()
    from psychopath_gb300 import scenes
    rays = scenes.incoherent_rays(P, F, 30000, seed=7)
    hg, ho, _, _ = _run(s, rays)
    st = sc.compare_hits(hg, ho)
    _assert_parity(st, 1000)


def test_grid_coherent(gpu_lib):
    s, P, F = sc.grid_small()
    from psychopath_gb300 import scenes
    rays = scenes.coherent_rays(128)
    hg, ho, _, _ = _run(s, rays)
    st = sc.compare_hits(hg, ho)
    _assert_parity(st, 5000)


def test_full_surface_data(gpu_lib):
    rays = sc.random_rays(5000, [-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], seed=5)
    hg, ho, fg, fo = _run(sc.cornell(), rays, full=True)
    same = (hg["kind"] >= abi.PSY_HIT_SURFACE) & (hg["kind"] == ho["kind"]) & (hg["prim"] == ho["prim"]) & (
        hg["inst"] == ho["inst"])
    assert same.sum() > 3000
    for f in ("pos", "nor", "nor_g"):
        np.testing.assert_allclose(fg[f][same], fo[f][same], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(fg["pos_err"][same], fo["pos_err"][same], rtol=1e-6)
    np.testing.assert_allclose(fg["sample_pdf"][same], fo["sample_pdf"][same], rtol=1e-4, atol=1e-7)
    assert np.array_equal(fg["shader"][same], fo["shader"][same])


@pytest.mark.parametrize("case", ["sphere", "motion"])
def test_fp16_bounds_conservative(gpu_lib, case):
    """FP16 outward-rounded child bounds lose no hit: results equal FP32's."""
    if case == "sphere":
        s = sc.sphere_small(level=5)
        rays = sc.targeted_rays(20000, [-1.1, -0.1, -1.1], [1.1, 2.1, 1.1], [-4, 0.05, -4], [4, 4, 4], seed=6)
    else:
        s = sc.motion_small()
        rays = sc.targeted_rays(20000, [-50, -50, -50], [50, 50, 50], [-60, -60, 60], [60, 60, 95], seed=8,
                                time_random=True)
    g32 = gpu.Scene(s)
    g16 = gpu.Scene(s, bounds="fp16")
    h32 = gpu.Tracer(g32).trace(rays)
    h16 = gpu.Tracer(g16).trace(rays)
    st = sc.compare_hits(h16, h32)
    _assert_parity(st, 100)


def test_empty_batch_and_misses(gpu_lib):
    s = sc.cornell()
    g = gpu.Scene(s)
    tr = gpu.Tracer(g)
    h = tr.trace(np.zeros(0, dtype=abi.ray_dtype()))
    assert len(h) == 0
    # rays leaving through the open front face miss everything
    from psychopath_gb300 import scenes
    rays = scenes.rays_array(np.array([[0, 1, 0.5]] * 4, dtype=np.float32),
                             np.array([[0, 0, 1], [0.01, 0, 1], [0, 0.01, 1], [0.1, 0.1, 1]], dtype=np.float32))
    h = tr.trace(rays)
    assert (h["kind"] == abi.PSY_HIT_MISS).all()


@pytest.mark.parametrize("mode,minb", [(0, 4), (0, 5), (0, 6), (0, 8), (1, 4), (1, 6), (1, 8), (2, 4), (3, 8)])
def test_trace_kernel_variants_identical(gpu_lib, mode, minb):
    """Every traversal kernel variant (one thread per ray, persistent with lane
    refill at each register budget, warp packets) returns identical hits."""
    s = sc.motion_small()
    rays = sc.targeted_rays(20000, [-50, -50, -50], [50, 50, 50], [-60, -60, 60], [60, 60, 95], seed=9,
                            time_random=True)
    g = gpu.Scene(s)
    tr = gpu.Tracer(g)
    g.set_trace(0, 4)
    ref = tr.trace(rays)
    g.set_trace(mode, minb)
    h = tr.trace(rays)
    assert np.array_equal(h, ref)


@pytest.mark.parametrize("mode,minb", [(0, 4), (0, 8), (1, 8), (2, 4), (3, 10), (5, 10)])
def test_binned_ray_order_identical(gpu_lib, mode, minb):
    """Sorting a large batch by two-point key only changes which thread
    traces which ray: hits are identical to the given order."""
    sd, P, F = sc.grid_small(256, 128)
    rays = np.concatenate([scenes.incoherent_rays(P, F, 1 << 16, seed=7), scenes.coherent_rays(128)])
    g = gpu.Scene(sd)
    tr = gpu.Tracer(g)
    g.set_trace(mode, minb)
    ref = tr.trace(rays)
    g.set_ray_order(True)
    h = tr.trace(rays)
    assert np.array_equal(h, ref)
    # a motion scene through the full-output kernel
    s = sc.motion_small()
    rays = sc.targeted_rays(70000, [-50, -50, -50], [50, 50, 50], [-60, -60, 60], [60, 60, 95], seed=3,
                            time_random=True)
    g2 = gpu.Scene(s, ray_order="binned")
    a, fa = gpu.Tracer(g2).trace(rays, full=True)
    g2.set_ray_order(False)
    b, fb = gpu.Tracer(g2).trace(rays, full=True)
    assert np.array_equal(a, b) and np.array_equal(fa, fb)


@pytest.mark.parametrize("n", [1, 4095, 4097, 70000, 300001, 4200001])
def test_ray_order_is_a_stable_sort(gpu_lib, n):
    """The ray order of binned trace calls: a permutation of the rays whose
    keys are non-decreasing, equal keys in their original order (the radix
    sort is stable); ragged sizes around the 4096-key tile, and 1026 tiles
    (the digit-row scan runs in chunks of 1024 tiles)."""
    sd, P, F = sc.grid_small(64, 32)
    rays = np.concatenate([scenes.incoherent_rays(P, F, n // 2, seed=5), scenes.coherent_rays(256)])[:n]
    if len(rays) < n:
        rays = np.concatenate([rays, scenes.incoherent_rays(P, F, n - len(rays), seed=6)])
    g = gpu.Scene(sd)
    keys, order = g.ray_order(rays)
    assert len(order) == n
    assert np.array_equal(np.sort(order), np.arange(n, dtype=np.uint32))
    assert (keys < (1 << 30)).all() and (np.diff(keys.astype(np.int64)) >= 0).all()
    tie = np.diff(keys.astype(np.int64)) == 0
    assert (np.diff(order.astype(np.int64))[tie] > 0).all()
    # a batch whose rays all share one key keeps the given order
    same = np.repeat(rays[:1], min(n, 5000))
    k2, o2 = g.ray_order(same)
    assert (k2 == k2[0]).all() and np.array_equal(o2, np.arange(len(same), dtype=np.uint32))
    g.close()


@pytest.mark.parametrize("case", ["grid", "motion", "cornell"])
def test_warp_packets_match_per_ray(gpu_lib, case):
    """Warp-packet traversal (octant groups per warp, split again at
    instance entry) gives bit-identical hits to one thread per ray, with
    mixed-octant warps, motion-blurred instances, lights and occlusion rays."""
    if case == "grid":
        sd, P, F = sc.grid_small(128, 64)
        rays = np.concatenate([scenes.incoherent_rays(P, F, 20000, seed=3), scenes.coherent_rays(100)])
    elif case == "motion":
        sd = sc.motion_small()
        rays = sc.targeted_rays(30000, [-50, -50, -50], [50, 50, 50], [-60, -60, 60], [60, 60, 95], seed=4,
                                time_random=True)
    else:
        sd = sc.cornell()
        rays = sc.random_rays(30000, [-1.0, 0.0, -1.0], [1.0, 2.0, 1.0], seed=5, occl_frac=0.5, max_t=1.5)
    g = gpu.Scene(sd)
    tr = gpu.Tracer(g)
    g.set_trace(0, 4)
    ref = tr.trace(rays)
    g.set_trace(2, 4)
    h = tr.trace(rays)
    assert np.array_equal(h, ref)
    g.counters(True)
    g.set_trace(2, 4)
    tr.trace(rays)
    pn, pt, _ = g.counters(False)
    g.counters(True)
    g.set_trace(0, 4)
    tr.trace(rays)
    rn, rt, _ = g.counters(False)
    assert (pn, pt) == (rn, rt)  # same node and triangle tests per ray


@pytest.mark.parametrize("mode,minb", [(3, 6), (3, 8), (3, 10), (3, 12), (5, 10)])
@pytest.mark.parametrize("bounds", ["fp32", "fp16"])
def test_static_scene_traversal_identical(gpu_lib, mode, minb, bounds):
    """The static-scene traversal (trace mode 3) and its lane-refill form
    (mode 5) return the same hits, bit for bit, as the general kernel on
    static scenes: closest and any hit, finite max_t, axis-parallel rays (the
    unordered slab test), the full surface output, and misses; with FP32 and
    with FP16 child bounds."""
    cases = []
    sd, P, F = sc.grid_small(256, 128)
    cases.append((sd, np.concatenate([scenes.incoherent_rays(P, F, 1 << 15, seed=7), scenes.coherent_rays(96)])))
    s = sc.sphere_small(level=4)
    cases.append((s, sc.targeted_rays(20000, [-1.1, -0.1, -1.1], [1.1, 2.1, 1.1], [-4, 0.05, -4], [4, 4, 4], seed=5)))
    rays = sc.random_rays(20000, [-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], seed=6, occl_frac=0.3)
    rays["max_t"][1::5] = 0.7
    ax = rays[::7].copy()  # axis-parallel directions: zero direction components
    ax["dir"][:, 0] = 0.0
    ax["dir"][:, 2] = 0.0
    ax["dir"][:, 1] = np.where(np.arange(len(ax)) % 2 == 0, 1.0, -1.0).astype(np.float32)
    cases.append((sc.cornell(), np.concatenate([rays, ax])))
    n_static = 0
    for sd, rays in cases:
        g = gpu.Scene(sd, bounds=bounds)
        n_static += g.flags()["static_fast"]
        tr = gpu.Tracer(g)
        g.set_trace(0, 4)
        ref, fref = tr.trace(rays, full=True)
        ref2 = tr.trace(rays)
        g.set_trace(mode, minb)
        h = tr.trace(rays)
        h2, f2 = tr.trace(rays, full=True)
        assert np.array_equal(h, ref2)
        assert np.array_equal(h2, ref) and np.array_equal(f2, fref)
        g.close()
    assert n_static >= 2  # the grid and the sphere scenes qualify


@pytest.mark.parametrize("minb", [8, 10])
def test_speculative_traversal_differs_only_at_ties(gpu_lib, minb):
    """The speculative static-scene traversal (trace mode 4) tests the same
    leaves in the same order plus, at times, nodes and triangles the
    reference culls after a hit; the closest hit may then differ only where
    a second triangle lies at exactly the same t.  Shadow rays do not
    speculate and are identical."""
    sd, P, F = sc.grid_small(256, 128)
    rays = np.concatenate([scenes.incoherent_rays(P, F, 1 << 15, seed=7), scenes.coherent_rays(96)])
    cases = [(sd, rays),
             (sc.sphere_small(level=4),
              sc.targeted_rays(20000, [-1.1, -0.1, -1.1], [1.1, 2.1, 1.1], [-4, 0.05, -4], [4, 4, 4], seed=5)),
             (sc.cornell(), sc.random_rays(20000, [-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], seed=6, occl_frac=0.3))]
    for sd, rays in cases:
        g = gpu.Scene(sd)
        tr = gpu.Tracer(g)
        g.set_trace(0, 4)
        ref = tr.trace(rays)
        g.set_trace(4, minb)
        h = tr.trace(rays)
        assert np.array_equal(h["kind"], ref["kind"])
        occ = (rays["flags"] & abi.PSY_RAY_OCCLUSION) != 0
        assert np.array_equal(h[occ], ref[occ])
        diff = h["prim"] != ref["prim"]
        assert np.array_equal(h["t"][diff], ref["t"][diff])  # only exact ties
        assert diff.mean() < 1e-3
        same = ~diff
        assert np.array_equal(h[same], ref[same])
        g.close()


def test_deep_tree_large_stack_kernels(gpu_lib):
    """A scene whose worst-case stack needs the 192-entry kernels: hits agree
    with the oracle, and the general and static-scene kernels at every
    register budget return identical hits."""
    s = sc.deep_stack()
    # rays from random origins toward random triangles' centroids
    rng = np.random.default_rng(12)
    cents = np.concatenate([od["verts"][0][od["indices"]].mean(axis=1) for od in s.objects])
    tgt = cents[rng.integers(0, len(cents), 20000)]
    org = rng.uniform([-1, -1, 2], [2, 4, 4], (20000, 3))
    rays = scenes.rays_array(org.astype(np.float32), (tgt - org).astype(np.float32))
    rays["flags"][::4] = abi.PSY_RAY_OCCLUSION
    hg, ho, _, _ = _run(s, rays)
    _assert_parity(sc.compare_hits(hg, ho), 2000)
    g = gpu.Scene(s)
    assert g.info()["stack_variant"] == 192 and g.flags()["static_fast"]
    tr = gpu.Tracer(g)
    g.set_trace(0, 4)
    ref = tr.trace(rays)
    for mode, minb in [(0, 8), (3, 6), (3, 8), (3, 10), (3, 12), (1, 8), (5, 10)]:
        g.set_trace(mode, minb)
        assert np.array_equal(tr.trace(rays), ref), (mode, minb)
    g.close()
