"""Small seeded scenes and ray sets shared by the parity tests (sizes the CPU
oracle finishes in seconds)."""
import math

import numpy as np

from psychopath_gb300 import abi, scenes


def cornell(w=32, h=32, spp=4, bounces=2):
    return scenes.cornell_box(w, h, spp, max_bounces=bounces)


def sphere_small(w=32, h=18, spp=4, bounces=6, level=4):
    return scenes.mesh_stress(w, h, spp, max_bounces=bounces, level=level)


def motion_small(w=32, h=18, spp=4, bounces=2, n=40, level=3, lights=8):
    return scenes.motion_instances(w, h, spp, max_bounces=bounces, n_instances=n, level=level, n_lights=lights)


def cornell_lens(w=32, h=32, spp=8, bounces=2):
    """The Cornell box seen through a thin lens with a moving camera: 3
    camera keys (the eye moves and turns), 2 field-of-view keys, 2 aperture
    radii and 2 focus distances, all lerped by the sample time
    (Camera::generate_ray, src/camera.rs:74-102)."""
    s = scenes.cornell_box(w, h, spp, max_bounces=bounces)
    keys = [scenes.look_at((0.25 * k - 0.25, 1.0 + 0.05 * k, 3.9 - 0.2 * k), (0.1 * k, 1.0, 0.0)) for k in range(3)]
    s.set_camera(keys, [40.0, 46.0], aperture_radii=[0.06, 0.1], focus_distances=[3.2, 4.1])
    return s


def flat_grid_edges(n=8):
    """A flat n x n grid of unit quads at y = 0 (2 triangles each) with
    integer vertex coordinates, and rays straight down through its vertices,
    edge midpoints and diagonal midpoints: the edge functions of the
    watertight test are exactly zero there, so the f64 retest
    (src/surface/triangle.rs:82-86) runs, and shared edges must still give
    exactly one closest hit."""
    xs = np.arange(n + 1, dtype=np.float64)
    X, Z = np.meshgrid(xs, xs)
    P = np.stack([X.ravel(), np.zeros(X.size), Z.ravel()], 1)
    ii = np.arange(n)[:, None] * (n + 1) + np.arange(n)[None, :]
    a, b, c, d = ii, ii + 1, ii + n + 2, ii + n + 1
    f = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)], 0)
    s = scenes.SceneData(16, 16, 1, 0, 2)
    sh = s.add_shader(abi.PSY_SHADER_LAMBERT, (0.7, 0.7, 0.7))
    s.add_instance(s.add_mesh(P, f.astype(np.uint32)), sh)
    s.set_camera([scenes.look_at((n / 2, 5.0, n / 2 + 5.0), (n / 2, 0.0, n / 2))], [50.0])
    pts = []
    for i in range(n + 1):
        for j in range(n + 1):
            pts.append((i, j))                  # vertices (incl. the border)
            if i < n:
                pts.append((i + 0.5, j))        # edges along x
            if j < n:
                pts.append((i, j + 0.5))        # edges along z
            if i < n and j < n:
                pts.append((i + 0.5, j + 0.5))  # the quads' diagonals
    pts = np.array(pts, dtype=np.float32)
    o = np.stack([pts[:, 0], np.full(len(pts), 3.0, np.float32), pts[:, 1]], 1)
    dirs = np.tile(np.array([[0.0, -1.0, 0.0]], np.float32), (len(pts), 1))
    return s, scenes.rays_array(o, dirs)


def grid_small(nx=64, ny=32):
    return scenes.grid_mesh(nx, ny)


def deep_stack(n_obj=24, seed=1):
    """Objects whose BVHs are as deep as the build allows: each mesh is 60
    clusters of 8 triangles at geometrically shrinking sizes and spacing, and
    the objects themselves sit at geometrically shrinking offsets, so the
    worst-case traversal stack (instance BVH + marker + mesh BVH) exceeds 64
    entries and the 192-entry kernels run.  Static, untransformed meshes."""
    rng = np.random.default_rng(seed)
    s = scenes.SceneData(16, 16, 1, seed, 2)
    sh = s.add_shader(abi.PSY_SHADER_LAMBERT, (0.7, 0.7, 0.7))
    for m in range(n_obj):
        off = np.array([0.0, 3.0 * (1.0 - 1.5 ** (-m)), 0.0])
        scale = 0.3 * 1.5 ** (-m)
        P, F = [], []
        for k in range(60):
            c, sz = 1.0 - 1.5 ** (-k), 0.2 * 1.5 ** (-k)
            for _ in range(8):
                p0 = np.array([c, 0.0, 0.0]) + rng.uniform(-sz, sz, 3)
                P += [p0, p0 + [sz * 0.3, 0.0, 0.0], p0 + [0.0, sz * 0.3, 0.0]]
                F.append([len(P) - 3, len(P) - 2, len(P) - 1])
        s.add_instance(s.add_mesh(np.array(P) * scale + off, np.array(F, dtype=np.uint32)), sh)
    s.set_camera([scenes.look_at((0.5, 1.5, 6.0), (0.5, 1.5, 0.0))], [50.0])
    return s


def random_rays(n, lo, hi, seed, time_random=False, occl_frac=0.0, max_t=None):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    r = scenes.rays_array(o, d)
    if time_random:
        r["time"] = rng.random(n).astype(np.float32)
        r["time"][:8] = np.array([0.0, 1.0, 0.5, 0.25, 0.75, 1.0, 0.0, 0.999], dtype=np.float32)
    if occl_frac > 0:
        r["flags"] = (rng.random(n) < occl_frac).astype(np.uint32) * abi.PSY_RAY_OCCLUSION
    if max_t is not None:
        r["max_t"] = rng.uniform(0.0, max_t, n).astype(np.float32)
    return r


def targeted_rays(n, targets_lo, targets_hi, origins_lo, origins_hi, seed, time_random=False):
    """Rays from random origins toward random targets (most of them hit)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(origins_lo, origins_hi, (n, 3))
    t = rng.uniform(targets_lo, targets_hi, (n, 3))
    d = (t - o)
    r = scenes.rays_array(o.astype(np.float32), d.astype(np.float32))
    if time_random:
        r["time"] = rng.random(n).astype(np.float32)
    return r


def compare_hits(hg, ho, near_edge_eps=1e-4):
    """Returns a dict of agreement statistics between GPU (hg) and oracle (ho)
    PsyHit arrays.  Mismatched primitive ids are allowed only at near-edge
    hits (a barycentric below near_edge_eps) or exact t ties."""
    kind_ok = hg["kind"] == ho["kind"]
    surf = (ho["kind"] >= abi.PSY_HIT_SURFACE) & kind_ok
    same_prim = (hg["prim"] == ho["prim"]) & (hg["inst"] == ho["inst"])
    t_o = ho["t"].astype(np.float64)
    t_g = hg["t"].astype(np.float64)
    rel = np.abs(t_g - t_o) / np.maximum(np.abs(t_o), 1e-30)
    bmin_o = np.minimum(np.minimum(ho["b0"], ho["b1"]), ho["b2"])
    bmin_g = np.minimum(np.minimum(hg["b0"], hg["b1"]), hg["b2"])
    near_edge = (np.abs(bmin_o) < near_edge_eps) | (np.abs(bmin_g) < near_edge_eps)
    tie = rel <= 1e-6
    unexplained = surf & ~same_prim & ~(near_edge | tie)
    return {
        "n": len(ho),
        "kind_mismatch": int((~kind_ok).sum()),
        "surface": int(surf.sum()),
        "prim_mismatch": int((surf & ~same_prim).sum()),
        "unexplained": int(unexplained.sum()),
        "t_max_rel": float(rel[surf & same_prim].max()) if (surf & same_prim).any() else 0.0,
        "t_bit_exact": float(np.mean(hg["t"][surf & same_prim] == ho["t"][surf & same_prim])) if (surf & same_prim).any() else 1.0,
        "occluded": int((ho["kind"] == abi.PSY_HIT_OCCLUDE).sum()),
    }
