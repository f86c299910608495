"""The oracle against the known answers of the reference's own unit tests
(each cites the reference test it repeats) and against independent Python
restatements of the integer hashes, the samplers' hash branch, the
wavelength mapping and the traversal table generator."""
import ctypes as C
import os

import numpy as np
import pytest

F12 = C.c_float * 12
F3 = C.c_float * 3


def xf(*v):
    return F12(*v)


def test_transform_multiply_kat(oracle_lib):
    # sub_crates/math3d/src/transform.rs:153-166 (multiply_test)
    a = xf(1.0, 2.0, 2.0, 1.5, 3.0, 6.0, 7.0, 8.0, 9.0, 2.0, 11.0, 12.0)
    b = xf(1.0, 5.0, 9.0, 13.0, 2.0, 6.0, 10.0, 14.0, 3.0, 7.0, 11.0, 15.0)
    out = F12()
    oracle_lib.psyo_xf_mul(a, b, out)
    assert list(out) == [97.0, 50.0, 136.0, 162.5, 110.0, 60.0, 156.0, 185.0, 123.0, 70.0, 176.0, 207.5]


def test_transform_inverse_kat(oracle_lib):
    # sub_crates/math3d/src/transform.rs:168-177 (inverse_test): a * a^-1 ~= identity (1e-7)
    a = xf(1.0, 0.33, 0.0, -2.0, 0.0, 1.0, 0.0, 0.0, 2.1, 0.7, 1.3, 0.0)
    inv, prod = F12(), F12()
    oracle_lib.psyo_xf_inverse(a, inv)
    oracle_lib.psyo_xf_mul(a, inv, prod)
    ident = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    for got, want in zip(prod, ident):
        assert abs(got - want) <= 1e-7 * max(1.0, abs(want)) + 1e-7


def test_point_matrix_kat(oracle_lib):
    # sub_crates/math3d/src/point.rs:166-184 (mul_matrix_1, mul_matrix_2)
    m = xf(1.0, 2.0, 2.0, 1.5, 3.0, 6.0, 7.0, 8.0, 9.0, 2.0, 11.0, 12.0)
    out = F3()
    oracle_lib.psyo_xf_point(m, F3(1.0, 2.5, 4.0), out)
    assert list(out) == [15.5, 54.0, 70.0]


def test_point_matrix_compose(oracle_lib):
    # sub_crates/math3d/src/point.rs:186-201 (mul_matrix_3): p * (m1 * m2) ~= (p * m1) * m2
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
    # src/lerp.rs:216-240 (lerp_matrix)
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


def test_vector_matrix_kat(oracle_lib):
    # sub_crates/math3d/src/vector.rs:220-236 (mul_matrix_1, mul_matrix_2)
    m = xf(1.0, 2.0, 2.0, 1.5, 3.0, 6.0, 7.0, 8.0, 9.0, 2.0, 11.0, 12.0)
    out = F3()
    oracle_lib.psyo_xf_vector(m, F3(1.0, 2.5, 4.0), out)
    assert list(out) == [14.0, 46.0, 58.0]


def test_normal_matrix_kat(oracle_lib):
    # sub_crates/math3d/src/normal.rs:209-220 (mul_matrix_1): within 4 ulps
    m = xf(1.0, 2.0, 2.0, 1.5, 3.0, 6.0, 7.0, 8.0, 9.0, 2.0, 11.0, 12.0)
    out = F3()
    oracle_lib.psyo_xf_normal(m, F3(1.0, 2.5, 4.0), out)
    for got, want in zip(out, (-4.0625, 1.78125, -0.03125)):
        g, w = np.float32(got).view(np.int32), np.float32(want).view(np.int32)
        assert abs(int(g) - int(w)) <= 4, (got, want)


@pytest.mark.parametrize("alpha,want", [(0.0, 1.0), (1.0, 2.0), (0.5, 1.5)])
def test_lerp_kat(oracle_lib, alpha, want):
    # src/lerp.rs:141-166 (lerp1, lerp2, lerp3)
    assert oracle_lib.psyo_lerp(1.0, 2.0, alpha) == want


@pytest.mark.parametrize("alpha,want", [(0.0, (1.0, 2.0, 1.0)), (1.0, (-2.0, 1.0, -1.0)), (0.5, (-0.5, 1.5, 0.0))])
def test_lerp_point_normal_vector_kat(oracle_lib, alpha, want):
    # src/lerp.rs:242-321 (lerp_point_*, lerp_normal_*, lerp_vector_*: one
    # storage type and one lerp for all three here, as in math3d over glam)
    out = F3()
    oracle_lib.psyo_lerp3(F3(1.0, 2.0, 1.0), F3(-2.0, 1.0, -1.0), alpha, out)
    assert tuple(out) == want


@pytest.mark.parametrize("alpha,want", [(0.0, 0.0), (1.0, 4.0), (0.5, 2.0), (0.25, 1.0), (0.75, 3.0), (0.625, 2.5)])
def test_lerp_slice_kat(oracle_lib, alpha, want):
    # src/lerp.rs:166-214 (lerp_slice1 .. lerp_slice6)
    s = (C.c_float * 5)(0.0, 1.0, 2.0, 3.0, 4.0)
    assert oracle_lib.psyo_lerp_slice(s, 5, alpha) == want


def test_ulp_kats(oracle_lib):
    # src/fp_utils.rs:88-130 (inc_ulp, dec_ulp, inc_ulp_zero, dec_ulp_zero, inc_dec_ulp, dec_inc_ulp)
    assert oracle_lib.psyo_increment_ulp_check() == 1


def test_hilbert_reversible(oracle_lib):
    # src/hilbert.rs:69-76 (reversible; d = 54 and more)
    x, y = C.c_uint32(), C.c_uint32()
    for d in (54, 0, 1, 7, 1000, 65535):
        oracle_lib.psyo_hilbert_d2xy(d, C.byref(x), C.byref(y))
        assert oracle_lib.psyo_hilbert_xy2d(x.value, y.value) == d


@pytest.mark.parametrize("place", [5, 3, 0, 9])
def test_quick_select(oracle_lib, place):
    # src/algorithm.rs:324-350 (quick_select_1 .. quick_select_4)
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


def _golden_ratio_sample(i, scramble):
    # src/renderer.rs:728-737
    n = ((i + _hash_u32(scramble, 0)) * 2654435769) & 0xFFFFFFFF
    return np.float32(np.float32(n) * np.float32(1.0 / 4294967296.0))


def _wavelengths(si, x, y, seed):
    # render_job's hero wavelength (src/renderer.rs:261-265) and
    # wavelengths() (src/color.rs:20-43), in f32 steps
    g = _golden_ratio_sample(si, _hash_u32(((x << 16) ^ y) & 0xFFFFFFFF, seed))
    hero = np.float32(g * np.float32(320.0)) + np.float32(380.0)
    out = []
    for k in range(4):
        wl = np.float32(hero + np.float32(np.float32(80.0) * np.float32(k)))
        out.append(np.float32(wl - np.float32(320.0)) if wl > np.float32(700.0) else wl)
    return np.array(out, dtype=np.float32)


def _sample_4d_hash_branch(i, dset, px, py, seed):
    # get_sample_4d for dimension sets past the Sobol sets (src/renderer.rs:714-723)
    s = (px ^ ((py << 16) & 0xFFFFFFFF) ^ ((seed * 0x736caf6f) & 0xFFFFFFFF)) & 0xFFFFFFFF
    return np.array([np.float32(np.float32(_hash_u32(((dset * 4 + k) ^ ((i << 16) & 0xFFFFFFFF)) & 0xFFFFFFFF, s))
                                * np.float32(1.0 / 4294967296.0)) for k in range(4)], dtype=np.float32)


def test_golden_ratio_and_wavelength(oracle_lib):
    for i in range(64):
        for scr in (0, 1, 0xdeadbeef):
            assert oracle_lib.psyo_golden_ratio_sample(i, scr) == _golden_ratio_sample(i, scr)
    out = (C.c_float * 4)()
    rng = np.random.default_rng(11)
    for si, x, y, seed in rng.integers(0, [4096, 4096, 4096, 2 ** 32], size=(300, 4)):
        oracle_lib.psyo_wavelengths(int(si), int(x), int(y), int(seed), out)
        assert np.array_equal(np.array(list(out), dtype=np.float32), _wavelengths(int(si), int(x), int(y), int(seed)))


def test_sample_4d_hash_branch(oracle_lib):
    out = (C.c_float * 4)()
    rng = np.random.default_rng(12)
    for i, dset, px, py, seed in rng.integers(0, [65536, 64, 4096, 4096, 2 ** 32], size=(300, 5)):
        dset = int(dset) + 2  # sets 0 and 1 are Sobol-Burley
        oracle_lib.psyo_get_sample_4d(int(i), dset, int(px), int(py), int(seed), out)
        want = _sample_4d_hash_branch(int(i), dset, int(px), int(py), int(seed))
        assert np.array_equal(np.array(list(out), dtype=np.float32), want)


def traversal_table_restated():
    """The traversal table of sub_crates/bvh_order/build.rs:17-76: for each
    ray octant, 27 four-child rows (split axes s0 top, s1 left, s2 right),
    9 + 9 three-child rows (left-heavy, right-heavy) and 3 two-child rows;
    each entry packs a child permutation 2 bits per position."""
    table = []
    for rd in range(8):
        ray = [rd & 1, (rd >> 1) & 1, (rd >> 2) & 1]
        row = []
        for s2 in range(3):
            for s1 in range(3):
                for s0 in range(3):
                    p = [0, 1, 2, 3]
                    if ray[s1]:
                        p[0], p[1] = p[1], p[0]
                    if ray[s2]:
                        p[2], p[3] = p[3], p[2]
                    if ray[s0]:
                        p = [p[2], p[3], p[0], p[1]]
                    row.append(p[0] + (p[1] << 2) + (p[2] << 4) + (p[3] << 6))
        for s1 in range(3):
            for s0 in range(3):
                p = [0, 1, 2]
                if ray[s1]:
                    p[0], p[1] = p[1], p[0]
                if ray[s0]:
                    p[0], p[1] = p[1], p[0]
                    p[0], p[2] = p[2], p[0]
                row.append(p[0] + (p[1] << 2) + (p[2] << 4))
        for s1 in range(3):
            for s0 in range(3):
                p = [0, 1, 2]
                if ray[s1]:
                    p[1], p[2] = p[2], p[1]
                if ray[s0]:
                    p[0], p[2] = p[2], p[0]
                    p[0], p[1] = p[1], p[0]
                row.append(p[0] + (p[1] << 2) + (p[2] << 4))
        for s0 in range(3):
            p = [0, 1]
            if ray[s0]:
                p[0], p[1] = p[1], p[0]
            row.append(p[0] + (p[1] << 2))
        table.append(row)
    return np.array(table, dtype=np.uint8)


def test_traversal_table(oracle_lib):
    # equals the generator's table, entry for entry
    t = (C.c_uint8 * (8 * 48))()
    oracle_lib.psyo_traversal_table(t)
    t = np.frombuffer(t, dtype=np.uint8).reshape(8, 48)
    assert np.array_equal(t, traversal_table_restated())
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
    """Regenerates the spectral tables from the reference's source file when
    PSY_REFERENCE_ROOT names a checkout of the reference (skipped otherwise)."""
    root = os.environ.get("PSY_REFERENCE_ROOT", "")
    src = os.path.join(root, "sub_crates", "spectral_upsampling", "src", "meng", "meng_spectra_tables.rs")
    if not root or not os.path.exists(src):
        pytest.skip("PSY_REFERENCE_ROOT not set to a reference checkout")
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
