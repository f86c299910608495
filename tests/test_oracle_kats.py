"""The oracle against the known answers of the reference's own unit tests
(and independent Python restatements of the integer hashes)."""
import ctypes as C
import os

import numpy as np
import pytest

F12 = C.c_float * 12
F3 = C.c_float * 3


def xf(*v):
    return F12(*v)


def test_transform_multiply_kat(oracle_lib):
    # sub_crates/math3d/src/transform.rs:181-194
    a = xf(1.0, 2.0, 2.0, 1.5, 3.0, 6.0, 7.0, 8.0, 9.0, 2.0, 11.0, 12.0)
    b = xf(1.0, 5.0, 9.0, 13.0, 2.0, 6.0, 10.0, 14.0, 3.0, 7.0, 11.0, 15.0)
    out = F12()
    oracle_lib.psyo_xf_mul(a, b, out)
    assert list(out) == [97.0, 50.0, 136.0, 162.5, 110.0, 60.0, 156.0, 185.0, 123.0, 70.0, 176.0, 207.5]


def test_transform_inverse_kat(oracle_lib):
    # sub_crates/math3d/src/transform.rs:196-205: a * a^-1 ~= identity (1e-7)
    a = xf(1.0, 0.33, 0.0, -2.0, 0.0, 1.0, 0.0, 0.0, 2.1, 0.7, 1.3, 0.0)
    inv, prod = F12(), F12()
    oracle_lib.psyo_xf_inverse(a, inv)
    oracle_lib.psyo_xf_mul(a, inv, prod)
    ident = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    for got, want in zip(prod, ident):
        assert abs(got - want) <= 1e-7 * max(1.0, abs(want)) + 1e-7


def test_point_matrix_kat(oracle_lib):
    # sub_crates/math3d/src/point.rs:372-390
    m = xf(1.0, 2.0, 2.0, 1.5, 3.0, 6.0, 7.0, 8.0, 9.0, 2.0, 11.0, 12.0)
    out = F3()
    oracle_lib.psyo_xf_point(m, F3(1.0, 2.5, 4.0), out)
    assert list(out) == [15.5, 54.0, 70.0]


def test_point_matrix_compose(oracle_lib):
    # sub_crates/math3d/src/point.rs:392-407: p * (m1 * m2) ~= (p * m1) * m2
    m1 = xf(1.0, 2.0, 2.0, 1.5, 3.0, 6.0, 7.0, 8.0, 9.0, 2.0, 11.0, 12.0)
    m2 = xf(4.0, 1.0, 2.0, 3.5, 3.0, 6.0, 5.0, 2.0, 2.0, 2.0, 4.0, 12.0)
    p = F3(1.0, 2.5, 4.0)
    m12, a, b, c = F12(), F3(), F3(), F3()
    oracle_lib.psyo_xf_mul(m1, m2, m12)
    oracle_lib.psyo_xf_point(m12, p, a)
    oracle_lib.psyo_xf_point(m1, p, b)
    oracle_lib.psyo_xf_point(m2, b, c)
    assert sum((x - y) ** 2 for x, y in zip(a, c)) <= 1e-5


def test_lerp_matrix_kat(oracle_lib):
    # src/lerp.rs:526-550
    a = xf(0.0, 2.0, 2.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 10.0, 11.0)
    b = xf(-1.0, 1.0, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 10.0, 11.0, 12.0)
    expect = {0.25: [-0.25, 1.75, 2.25, 3.25, 4.25, 5.25, 6.25, 7.25, 8.25, 9.25, 10.25, 11.25],
              0.5: [-0.5, 1.5, 2.5, 3.5, 4.5, 5.5, 6.5, 7.5, 8.5, 9.5, 10.5, 11.5],
              0.75: [-0.75, 1.25, 2.75, 3.75, 4.75, 5.75, 6.75, 7.75, 8.75, 9.75, 10.75, 11.75]}
    out = F12()
    oracle_lib.psyo_xf_lerp(a, b, 0.0, out)
    assert list(out) == list(a)
    oracle_lib.psyo_xf_lerp(a, b, 1.0, out)
    assert list(out) == list(b)
    for al, e in expect.items():
        oracle_lib.psyo_xf_lerp(a, b, al, out)
        assert list(out) == e


@pytest.mark.parametrize("alpha,want", [(0.0, 0.0), (1.0, 4.0), (0.5, 2.0), (0.25, 1.0), (0.75, 3.0), (0.625, 2.5)])
def test_lerp_slice_kat(oracle_lib, alpha, want):
    # src/lerp.rs:478-524
    s = (C.c_float * 5)(0.0, 1.0, 2.0, 3.0, 4.0)
    assert oracle_lib.psyo_lerp_slice(s, 5, alpha) == want


def test_ulp_kats(oracle_lib):
    # src/fp_utils.rs:84-131
    assert oracle_lib.psyo_increment_ulp_check() == 1


def test_hilbert_reversible(oracle_lib):
    # src/hilbert.rs:65-77
    x, y = C.c_uint32(), C.c_uint32()
    for d in (54, 0, 1, 7, 1000, 65535):
        oracle_lib.psyo_hilbert_d2xy(d, C.byref(x), C.byref(y))
        assert oracle_lib.psyo_hilbert_xy2d(x.value, y.value) == d


@pytest.mark.parametrize("place", [5, 3, 0, 9])
def test_quick_select(oracle_lib, place):
    # src/algorithm.rs:307-351
    lst = (C.c_int32 * 10)(8, 9, 7, 4, 6, 1, 0, 5, 3, 2)
    assert oracle_lib.psyo_quick_select_ints(lst, 10, place) == place


def _hash_u32(n, seed):
    h = n
    for _ in range(3):
        h = (h * 0x736caf6f) & 0xFFFFFFFF
        h ^= h >> 16
        h ^= seed
    return h


def _hash_u64(n, seed):
    h = n
    k = (32416190071 * 314604959) & 0xFFFFFFFFFFFFFFFF
    for _ in range(4):
        h = (h * k) & 0xFFFFFFFFFFFFFFFF
        h ^= h >> 32
        h ^= seed
    return h


def test_hashes_bit_exact(oracle_lib):
    rng = np.random.default_rng(3)
    for n, s in rng.integers(0, 2 ** 32, size=(200, 2)):
        n, s = int(n), int(s)
        assert oracle_lib.psyo_hash_u32(n, s) == _hash_u32(n, s)
        assert oracle_lib.psyo_hash_u64(n * 7919, s) == _hash_u64(n * 7919, s)
        f = np.float32(np.float32(_hash_u32(n, s)) * np.float32(1.0 / 4294967296.0))
        assert oracle_lib.psyo_hash_u32_to_f32(n, s) == f


def test_golden_ratio_and_wavelength(oracle_lib):
    for i in range(64):
        for scr in (0, 1, 0xdeadbeef):
            n = ((i + _hash_u32(scr, 0)) * 2654435769) & 0xFFFFFFFF
            want = np.float32(np.float32(n) * np.float32(1.0 / 4294967296.0))
            assert oracle_lib.psyo_golden_ratio_sample(i, scr) == want


def test_traversal_table(oracle_lib):
    # sub_crates/bvh_order/build.rs: every row is a permutation of the children
    t = (C.c_uint8 * (8 * 48))()
    oracle_lib.psyo_traversal_table(t)
    t = np.frombuffer(t, dtype=np.uint8).reshape(8, 48)
    for rd in range(8):
        for k in range(27):
            assert sorted((t[rd, k] >> (2 * i)) & 3 for i in range(4)) == [0, 1, 2, 3]
        for k in range(27, 45):
            assert sorted((t[rd, k] >> (2 * i)) & 3 for i in range(3)) == [0, 1, 2]
        for k in range(45, 48):
            assert sorted((t[rd, k] >> (2 * i)) & 3 for i in range(2)) == [0, 1]
    # octant 0 never permutes
    assert t[0, 0] == 0 + (1 << 2) + (2 << 4) + (3 << 6)


def test_probit_center_and_tails(oracle_lib):
    from scipy.special import ndtri
    for v in (0.5, 0.1, 0.9, 0.01, 0.99, 0.3333):
        assert abs(oracle_lib.psyo_probit(v, 1.0) - ndtri(v)) < 1e-5
    assert oracle_lib.psyo_probit(0.5, 2.0 / 6.0) == 0.0


def test_fast_exp_accuracy(oracle_lib):
    for p in np.linspace(-60, 10, 200):
        got = oracle_lib.psyo_fast_exp(float(p))
        assert abs(got - np.exp(p)) <= 1e-4 * np.exp(p) + 1e-30


def test_spectrum_equal_energy_white(oracle_lib):
    # XYZ (1,1,1) upsamples to a flat spectrum of 1 (equal-energy reflectance)
    out = (C.c_float * 4)()
    for hero in (380.0, 450.0, 550.0, 699.0):
        oracle_lib.psyo_xyz_to_spectrum((C.c_float * 3)(1.0, 1.0, 1.0), hero, out)
        assert np.allclose(list(out), 1.0, atol=0.02)


def test_rec709_matrix_matches_python(oracle_lib):
    from psychopath_gb300 import scenes
    out = (C.c_float * 3)()
    for rgb in ((1, 0, 0), (0.2, 0.5, 0.9), (0.73, 0.73, 0.73)):
        oracle_lib.psyo_rec709_e_to_xyz((C.c_float * 3)(*rgb), out)
        assert list(out) == [float(v) for v in scenes.rec709_e_to_xyz(rgb)]


def test_triangle_watertight_shared_edge(oracle_lib):
    # rays through a shared edge hit exactly one of the two triangles or both
    # with the same t; never neither (watertightness)
    rng = np.random.default_rng(5)
    a, b, c, d = (0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (1.0, 1.0, 0.0)
    P = lambda v: (C.c_float * 3)(*v)
    out = (C.c_float * 4)()
    for _ in range(500):
        s = rng.random()
        target = (s, 1.0 - s, 0.0)  # on edge b-c
        o = (target[0] + rng.normal() * 0.3, target[1] + rng.normal() * 0.3, 1.0 + rng.random())
        dv = tuple(t - oo for t, oo in zip(target, o))
        h1 = oracle_lib.psyo_intersect_triangle(P(o), P(dv), float("inf"), P(a), P(b), P(c), out)
        h2 = oracle_lib.psyo_intersect_triangle(P(o), P(dv), float("inf"), P(b), P(d), P(c), out)
        assert h1 or h2


def test_meng_tables_match_reference():
    src = "/root/reference/sub_crates/spectral_upsampling/src/meng/meng_spectra_tables.rs"
    if not os.path.exists(src):
        pytest.skip("reference tree not present")
    import subprocess
    import sys
    import tempfile
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    gen = os.path.join(here, "psychopath_gb300", "csrc", "gen_spectra_tables.py")
    committed = os.path.join(here, "psychopath_gb300", "csrc", "spectra_tables.inc")
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "t.inc")
        subprocess.run([sys.executable, gen, src, out], check=True)
        assert open(out).read() == open(committed).read()
