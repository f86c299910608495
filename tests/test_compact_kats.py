"""The oracle's restatement of the `compact` crate (oracle/oracle_compact.cpp),
pinned on the CPU: every known answer of the crate's own unit and property
tests (tests/compact_cases.py), an independent numpy restatement of the
encoders on seeded inputs over the whole f32 range, numpy's IEEE binary16
conversion for the colour format's half factor, and the colour / closure
byte layouts of src/color.rs and src/shading/surface_closure.rs."""
import ctypes as C

import numpy as np
import pytest

import oracle
from psychopath_gb300 import abi
from tests import compact_cases as cc


@pytest.fixture(scope="module")
def B():
    return cc.OracleBackend(oracle.lib())


def test_fluv32_known_answers(B):
    cc.check_fluv32(B)


def test_oct32_known_answers_and_precision(B):
    cc.check_oct32(B)


def test_unsigned32_known_answers(B):
    cc.check_unsigned32(B)


def test_unsigned40_known_answers(B):
    cc.check_unsigned40(B)


def test_signed48_known_answers(B):
    cc.check_signed48(B)


def test_signed48_ignores_upper_bits():
    """signed48.rs garbage_upper_bits_decode: decode_64 masks bits 48..63."""
    L = oracle.lib()
    b = cc.OracleBackend(L)
    for t in ((4.0, -623.53, 12.3), (-63456254.2, 5235423.53, 54353.3), (-0.000000634, 0.00000000005, 0.00000000892)):
        n = cc.enc(b, cc.F["signed48"], t)
        a, g = (C.c_float * 3)(), (C.c_float * 3)()
        L.psyo_signed48_decode_u64(n, a)
        L.psyo_signed48_decode_u64(n | 0xffff_0000_0000_0000, g)
        assert list(a) == list(g)


def test_encoders_match_numpy_restatement(B):
    v = cc.random_triples(200_000, seed=5)
    codes, _ = B.encode(cc.F["fluv32"], v)
    assert np.array_equal(codes.view("<u4").reshape(-1), cc.np_fluv32_encode(v))
    codes, _ = B.encode(cc.F["oct32"], v)
    assert np.array_equal(codes.view("<u4").reshape(-1), cc.np_oct32_encode(v))
    for name, mbits, ebits, bias, signed in (("unsigned32", 9, 5, 11, False), ("unsigned40", 11, 7, 32, False),
                                             ("signed48", 13, 6, 26, True)):
        codes, _ = B.encode(cc.F[name], v)
        size = codes.shape[1]
        wide = np.zeros((codes.shape[0], 8), np.uint8)
        wide[:, :size] = codes
        assert np.array_equal(wide.view("<u8").reshape(-1), cc.np_shared_encode(v, mbits, ebits, bias, signed)), name


def test_invalid_counts_follow_the_debug_assertions(B):
    v = cc.random_triples(50_000, seed=6)
    neg_or_nan = int(np.sum(~np.all(v >= 0, axis=1)))
    nan = int(np.sum(np.any(np.isnan(v), axis=1)))
    assert neg_or_nan > 1000 and nan > 100
    for name, want in (("fluv32", neg_or_nan), ("unsigned32", neg_or_nan), ("unsigned40", neg_or_nan),
                       ("signed48", nan), ("oct32", 0), ("oct32_precise", 0)):
        assert B.encode(cc.F[name], v)[1] == want, name


def test_shared_exponent_decode_is_exact(B):
    """Decoding is lossless: re-encoding a decoded value gives the same code."""
    v = cc.random_triples(100_000, seed=7)
    for name in ("unsigned32", "unsigned40", "signed48"):
        fmt = cc.F[name]
        if name != "signed48":
            v = np.abs(v)
        codes, _ = B.encode(fmt, v)
        again, _ = B.encode(fmt, B.decode(fmt, codes))
        assert np.array_equal(codes, again), name


def test_oct32_decode_encode_round_trip(B):
    """oct32 codes that decode inside the octahedron re-encode to themselves."""
    codes = cc.random_codes(100_000, 4, seed=8)
    d = B.decode(cc.F["oct32"], codes)
    again, _ = B.encode(cc.F["oct32"], d)
    u = codes.view("<u4").reshape(-1)
    a = (u >> 16).astype(np.uint16).view(np.int16).astype(np.int64)
    b = (u & 0xffff).astype(np.uint16).view(np.int16).astype(np.int64)
    inside = (np.abs(a) + np.abs(b) < 32767 - 2) & (np.abs(a) <= 32767) & (np.abs(b) <= 32767)
    assert np.mean(again.view("<u4").reshape(-1)[inside] == u[inside]) > 0.999


def test_f16_matches_numpy():
    L = oracle.lib()
    rng = np.random.default_rng(9)
    vals = np.concatenate([(np.exp2(rng.uniform(-30, 18, 50_000)) * rng.choice([-1, 1], 50_000)).astype(np.float32),
                           np.asarray([0.0, -0.0, 65504.0, 65519.996, 65520.0, 1e9, -np.inf, np.inf, 2.0 ** -25,
                                       2.0 ** -24, 1.5 * 2.0 ** -25, 2.0 ** -26, 6.1035156e-05, 6.097555e-05],
                                      np.float32)])
    got = np.asarray([L.psyo_f16_from_f32(float(x)) for x in vals], np.uint16)
    with np.errstate(over="ignore"):
        assert np.array_equal(got, vals.astype(np.float16).view(np.uint16))
    assert L.psyo_f16_from_f32(float("nan")) & 0x7e00 == 0x7e00
    h = np.arange(65536, dtype=np.uint32).astype(np.uint16)
    ref = h.view(np.float16).astype(np.float32)
    back = np.asarray([L.psyo_f16_to_f32(int(x)) for x in h], np.float32)
    fin = ~np.isnan(ref)
    assert np.array_equal(back[fin].view(np.uint32), ref[fin].view(np.uint32))
    assert np.all(np.isnan(back[~fin]))


def _colors(rows):
    c = np.zeros(len(rows), abi.color_dtype())
    for i, (k, v) in enumerate(rows):
        c[i]["kind"] = k
        c[i]["v"] = v
    return c


def test_color_and_closure_byte_layout():
    L = oracle.lib()
    cols = _colors([(abi.PSY_COLOR_XYZ, (1.0, 1.0, 1.0)), (abi.PSY_COLOR_BLACKBODY, (6500.0, 2.0, 0.0)),
                    (abi.PSY_COLOR_TEMPERATURE, (70000.0, -1.0, 0.0)), (abi.PSY_COLOR_BLACKBODY, (-5.0, 0.0, 9.0))])
    out = np.zeros((4, 5), np.uint8)
    bad = C.c_uint32()
    assert L.psyo_color_compress(cols.ctypes.data, 4, out.ctypes.data, C.byref(bad)) == 0 and bad.value == 0
    assert out[0].tolist() == [0, 0xc3, 0x56, 0x00, 0x7e]  # fluv32 0x7e0056c3, native (little) endian
    assert out[1].tolist() == [1, 0x64, 0x19, 0x00, 0x40]  # 6500 = 0x1964, f16(2.0) = 0x4000
    assert out[2].tolist() == [2, 0xff, 0xff, 0x00, 0xbc]  # saturating u16, f16(-1.0) = 0xbc00
    assert out[3].tolist() == [1, 0x00, 0x00, 0x00, 0x00]
    back = np.zeros(4, abi.color_dtype())
    assert L.psyo_color_decompress(out.ctypes.data, 4, back.ctypes.data, C.byref(bad)) == 0 and bad.value == 0
    assert back["kind"].tolist() == [0, 1, 2, 1]
    assert back["v"][1].tolist() == [6500.0, 2.0, 0.0] and back["v"][2].tolist() == [65535.0, -1.0, 0.0]

    sh = np.zeros(3, abi.shader_dtype())
    sh[0]["kind"], sh[0]["color"] = abi.PSY_SHADER_LAMBERT, cols[0]
    sh[1]["kind"], sh[1]["color"], sh[1]["roughness"], sh[1]["fresnel"] = abi.PSY_SHADER_GGX, cols[1], 0.5, 2.0
    sh[2]["kind"], sh[2]["color"] = abi.PSY_SHADER_EMIT, cols[2]
    rec = np.zeros((3, 12), np.uint8)
    assert L.psyo_closure_compress(sh.ctypes.data, 3, 12, rec.ctypes.data, C.byref(bad)) == 0 and bad.value == 0
    assert rec[0, :6].tolist() == [0] + out[0].tolist()
    assert rec[1, :10].tolist() == [1, 0xff, 0x7f, 0xff, 0xff] + out[1].tolist()  # 0.5 -> 32767, 2.0 clamps to 1
    assert rec[2, :6].tolist() == [2] + out[2].tolist()
    dsh = np.zeros(3, abi.shader_dtype())
    assert L.psyo_closure_decompress(rec.ctypes.data, 3, 12, dsh.ctypes.data, C.byref(bad)) == 0 and bad.value == 0
    assert dsh["kind"].tolist() == [abi.PSY_SHADER_LAMBERT, abi.PSY_SHADER_GGX, abi.PSY_SHADER_EMIT]
    assert dsh[1]["roughness"] == np.float32(32767) * np.float32(1.0 / 65535.0) and dsh[1]["fresnel"] == 1.0
    # a GGX record does not fit a 6-byte stride: counted, left unwritten
    rec6 = np.full((3, 6), 0xee, np.uint8)
    assert L.psyo_closure_compress(sh.ctypes.data, 3, 6, rec6.ctypes.data, C.byref(bad)) == 0 and bad.value == 1
    assert rec6[1].tolist() == [0xee] * 6
    assert L.psyo_closure_compress(sh.ctypes.data, 3, 5, rec6.ctypes.data, C.byref(bad)) == -1
