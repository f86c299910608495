"""Generates the golden fixtures of the parity tests (tests/golden/*.npz)
from the CPU oracle on seeded inputs: per-ray hits on four scenes, a small
Cornell render, Halton samples of every dimension, hash values, golden-ratio
samples, get_sample_4d values (Sobol-Burley and hash sets) and the camera's
hero wavelengths.  The
reference (a Rust crate) cannot be built here, so the oracle -- pinned by
the reference's own unit-test answers (tests/test_oracle_kats.py) -- is the
source; the fixtures freeze its outputs so that a later change to the oracle
and to the GPU path in the same wrong way still fails.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import lib as oracle_lib  # noqa: E402
from oracle.runner import OracleScene  # noqa: E402
from psychopath_gb300 import abi, scenes  # noqa: E402
from tests import scene_cases as sc  # noqa: E402


def golden_ray_sets():
    """(name, scene, rays): the seeded inputs the fixtures cover."""
    out = []
    r = sc.random_rays(2000, [-0.95, 0.05, -0.95], [0.95, 1.95, 0.95], seed=101, occl_frac=0.25, max_t=3.0)
    out.append(("cornell", sc.cornell(), r))
    out.append(("sphere", sc.sphere_small(level=4),
                sc.targeted_rays(2000, [-1.1, -0.1, -1.1], [1.1, 2.1, 1.1], [-4, 0.05, -4], [4, 4, 4], seed=102)))
    sd, P, F = sc.grid_small()
    out.append(("grid", sd, scenes.incoherent_rays(P, F, 2000, seed=103)))
    out.append(("motion", sc.motion_small(),
                sc.targeted_rays(2000, [-50, -50, -50], [50, 50, 50], [-60, -60, 60], [60, 60, 95], seed=104,
                                 time_random=True)))
    return out


def golden_render_scene():
    return sc.cornell(16, 16, 4, 2)


HALTON_INDICES = np.array(list(range(48)) + [65535, 65536, 2 ** 31, 2 ** 32 - 1] +
                          [int(x) for x in np.random.default_rng(105).integers(0, 2 ** 32, 12)], dtype=np.uint32)


def golden_ratio_args():
    """(sample index, scramble) pairs of golden_ratio_sample."""
    rng = np.random.default_rng(106)
    a = [(i, s) for i in range(16) for s in (0, 1, 0xDEADBEEF)]
    a += [tuple(int(v) for v in r) for r in rng.integers(0, 2 ** 32, size=(64, 2))]
    return np.array(a, dtype=np.uint32)


def sample_4d_args():
    """(sample index, dimension set, px, py, seed) rows of get_sample_4d:
    the two Sobol-Burley sets the camera uses and hash-branch sets."""
    rng = np.random.default_rng(107)
    rows = []
    for dset in (0, 1, 2, 5, 31):
        for i in list(range(8)) + [int(v) for v in rng.integers(0, 65536, 8)]:
            px, py, seed = (int(v) for v in rng.integers(0, [4096, 4096, 2 ** 32]))
            rows.append((i, dset, px, py, seed))
    rows.append((0, 0, 0, 0, 0))
    rows.append((0xFFFFFFFF, 1, 4095, 4095, 0xFFFFFFFF))
    return np.array(rows, dtype=np.uint32)


def wavelength_args():
    """(sample index, x, y, seed) rows of the camera's 4 hero wavelengths."""
    rng = np.random.default_rng(108)
    rows = [(i, 0, 0, 0) for i in range(8)]
    rows += [tuple(int(v) for v in r) for r in rng.integers(0, [4096, 4096, 4096, 2 ** 32], size=(64, 4))]
    return np.array(rows, dtype=np.uint32)


def main():
    L = oracle_lib()
    for name, sd, rays in golden_ray_sets():
        hits, _, _, _ = OracleScene(sd).trace(rays, threads=1)
        np.savez_compressed(os.path.join(HERE, "hits_%s.npz" % name), rays=rays.view(np.uint8),
                            hits=hits.view(np.uint8))
    img, _ = OracleScene(golden_render_scene()).render(threads=1)
    np.savez_compressed(os.path.join(HERE, "render_cornell16.npz"), xyz=img)
    hal = np.zeros((128, len(HALTON_INDICES)), dtype=np.float32)
    v = C.c_float()
    for d in range(128):
        for j, i in enumerate(HALTON_INDICES):
            assert L.psyo_halton_sample(int(i), d, C.byref(v)) == 0
            hal[d, j] = v.value
    n = np.arange(0, 4096, 7, dtype=np.uint32)
    seeds = np.array([0, 1, 0x736CAF6F, 0xFFFFFFFF], dtype=np.uint32)
    h32 = np.array([[L.psyo_hash_u32(int(a), int(s)) for a in n] for s in seeds], dtype=np.uint32)
    hf = np.array([[L.psyo_hash_u32_to_f32(int(a), int(s)) for a in n] for s in seeds], dtype=np.float32)
    ga, gv = golden_ratio_args(), []
    for i, scr in ga:
        gv.append(L.psyo_golden_ratio_sample(int(i), int(scr)))
    s4a = sample_4d_args()
    s4v = np.zeros((len(s4a), 4), dtype=np.float32)
    out = (C.c_float * 4)()
    for r, (i, dset, px, py, seed) in enumerate(s4a):
        L.psyo_get_sample_4d(int(i), int(dset), int(px), int(py), int(seed), out)
        s4v[r] = list(out)
    wla = wavelength_args()
    wlv = np.zeros((len(wla), 4), dtype=np.float32)
    for r, (si, x, y, seed) in enumerate(wla):
        L.psyo_wavelengths(int(si), int(x), int(y), int(seed), out)
        wlv[r] = list(out)
    np.savez_compressed(os.path.join(HERE, "samplers.npz"), halton_indices=HALTON_INDICES, halton=hal,
                        hash_n=n, hash_seeds=seeds, hash_u32=h32, hash_u32_to_f32=hf,
                        golden_args=ga, golden=np.array(gv, dtype=np.float32), sample_4d_args=s4a,
                        sample_4d=s4v, wavelength_args=wla, wavelengths=wlv)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
