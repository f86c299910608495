"""The GPU library's compact codecs (psy_compact_*, psy_fluv32_decode_yuv,
psy_color_*, psy_closure_*) against the oracle: the `compact` crate's own
known answers through the GPU, bit-exact agreement with the oracle on seeded
inputs over the whole f32 range (ragged sizes, unaligned buffers, a
full-size batch larger than L2), and the crate-style Python interface."""
import numpy as np
import pytest

from psychopath_gb300 import abi, compact

from . import compact_cases as cc

pytestmark = pytest.mark.gpu


class GpuBackend:
    """The library's batch calls on device buffers; `offset` shifts both
    buffers off their 16-byte alignment (the byte-wise copy path)."""

    def __init__(self, offset=0):
        self.offset = offset

    def _dev(self, a):
        import torch
        raw = np.ascontiguousarray(a).reshape(-1).view(np.uint8)
        t = torch.zeros(raw.size + 16, dtype=torch.uint8, device="cuda")
        if raw.size:
            t[self.offset:self.offset + raw.size] = torch.from_numpy(raw.copy()).cuda()
        return t

    def _out(self, nbytes):
        import torch
        return torch.zeros(nbytes + 16, dtype=torch.uint8, device="cuda")

    def _get(self, t, nbytes):
        import torch
        torch.cuda.synchronize()
        return t[self.offset:self.offset + nbytes].cpu().numpy()

    def encode(self, fmt, xyz):
        import torch
        xyz = np.ascontiguousarray(np.asarray(xyz, np.float32).reshape(-1, 3))
        n, size = xyz.shape[0], cc.SIZE[fmt]
        d_in, d_out = self._dev(xyz), self._out(n * size)
        bad = torch.zeros(1, dtype=torch.int32, device="cuda")
        compact.encode_device(fmt, d_in.data_ptr() + self.offset, n, d_out.data_ptr() + self.offset, bad.data_ptr())
        return self._get(d_out, n * size).reshape(n, size), int(bad.item())

    def decode(self, fmt, codes):
        codes = np.ascontiguousarray(np.asarray(codes, np.uint8).reshape(-1, cc.SIZE[fmt]))
        n = codes.shape[0]
        d_in, d_out = self._dev(codes), self._out(12 * n)
        compact.decode_device(fmt, d_in.data_ptr() + self.offset, n, d_out.data_ptr() + self.offset)
        return self._get(d_out, 12 * n).view(np.float32).reshape(n, 3)

    def decode_yuv(self, codes):
        from psychopath_gb300.gpu import _check, lib
        codes = np.ascontiguousarray(np.asarray(codes, np.uint32).reshape(-1))
        n = codes.size
        d_in, d_out = self._dev(codes), self._out(8 * n)
        _check(lib().psy_fluv32_decode_yuv(d_in.data_ptr() + self.offset, n, d_out.data_ptr() + self.offset, None))
        r = self._get(d_out, 8 * n).view(abi.yuv_dtype())
        return r["y"], r["u"], r["v"]


@pytest.fixture(scope="module")
def O(oracle_lib):
    return cc.OracleBackend(oracle_lib)


@pytest.fixture(scope="module", autouse=True)
def _built(gpu_lib):
    return gpu_lib


def same_floats(a, b):
    """Bit-equal, except that any NaN matches any NaN (payloads are the
    hardware's: x86 and the GPU make different default NaNs)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all(both_nan | (a.view(np.uint32) == b.view(np.uint32))))


@pytest.mark.parametrize("check", ["fluv32", "oct32", "unsigned32", "unsigned40", "signed48"])
def test_known_answers_on_gpu(check):
    getattr(cc, "check_" + check)(GpuBackend())


@pytest.mark.parametrize("offset", [0, 1, 4, 8])
@pytest.mark.parametrize("n", [0, 1, 1023, 1024, 1025, 70_001])
def test_encode_decode_bit_exact(O, n, offset):
    G = GpuBackend(offset)
    v = cc.random_triples(n, seed=100 + n)
    for name, fmt in cc.F.items():
        gc, gb = G.encode(fmt, v)
        oc, ob = O.encode(fmt, v)
        assert np.array_equal(gc, oc), (name, n, offset)
        assert gb == ob, (name, n, offset)
        if name == "oct32_precise":
            continue
        codes = cc.random_codes(n, cc.SIZE[fmt], seed=200 + n)
        assert same_floats(G.decode(fmt, codes), O.decode(fmt, codes)), (name, n, offset)
        assert same_floats(G.decode(fmt, oc), O.decode(fmt, oc)), (name, n, offset)
    codes = cc.random_codes(n, 4, seed=300 + n).view("<u4").reshape(-1)
    gy, gu, gv = G.decode_yuv(codes)
    oy, ou, ov = O.decode_yuv(codes)
    assert same_floats(gy, oy) and np.array_equal(gu, ou) and np.array_equal(gv, ov)


def test_oct32_precise_near_ties(O):
    """Directions half-way between neighbouring oct32 grid points (and at
    grid points and corners) put two candidates within rounding of each
    other: the f32 pre-ranking must hand these to the f64 cosines and still
    pick the crate's candidate."""
    n = 200_000
    codes = cc.random_codes(n, 4, seed=31).view("<u4").reshape(-1)
    nxt = np.stack([codes, (codes & 0xffff0000) | ((codes + 1) & 0xffff), codes + 0x10000,
                    (codes + 0x10001) & 0xffffffff], 1)
    d = O.decode(cc.F["oct32"], nxt.reshape(-1, 1).view(np.uint8)).reshape(n, 4, 3)
    mids = np.concatenate([d[:, 0], (d[:, 0] + d[:, 1]) * np.float32(0.5), (d[:, 0] + d[:, 2]) * np.float32(0.5),
                           (d[:, 0] + d[:, 3]) * np.float32(0.5),
                           (d[:, 0] + d[:, 1] + d[:, 2] + d[:, 3]) * np.float32(0.25)]).astype(np.float32)
    mids = np.concatenate([mids, mids * np.float32(1e-20), mids * np.float32(3e25), mids * np.float32(1e-33)])
    fmt = cc.F["oct32_precise"]
    gc, _ = GpuBackend().encode(fmt, mids)
    oc, _ = O.encode(fmt, mids)
    assert np.array_equal(gc, oc)


def test_full_size_batch(O):
    """A batch larger than L2 (8M triples, 96 MB in, 32-48 MB out) agrees
    with the oracle bit for bit, and decode(encode(x)) re-encodes to the same
    code for the shared-exponent formats (decoding is exact)."""
    n = 8 * 1024 * 1024
    G = GpuBackend()
    v = cc.random_triples(n, seed=4242)
    for name in ("fluv32", "oct32", "unsigned32", "unsigned40", "signed48"):
        fmt = cc.F[name]
        gc, gb = G.encode(fmt, v)
        oc, ob = O.encode(fmt, v)
        assert np.array_equal(gc, oc) and gb == ob, name
        gd = G.decode(fmt, gc)
        assert same_floats(gd, O.decode(fmt, oc)), name
        if name in ("unsigned32", "unsigned40", "signed48"):
            again, _ = G.encode(fmt, gd)
            fin = ~np.any(np.isnan(v), axis=1) & (np.all(v >= 0, axis=1) | (name == "signed48"))
            assert np.array_equal(again[fin], gc[fin]), name


def _random_colors(n, rng):
    c = np.zeros(n, abi.color_dtype())
    c["kind"] = rng.choice([0, 0, 1, 2, 7], n)
    c["v"] = cc.random_triples(n, seed=int(rng.integers(1 << 30)))
    t = c["kind"] != 0
    c["v"][t, 0] = rng.uniform(-100.0, 80000.0, int(t.sum())).astype(np.float32)
    return c


def test_color_and_closure_bit_exact(oracle_lib):
    import ctypes as C
    import torch
    from psychopath_gb300.gpu import _check, lib
    rng = np.random.default_rng(77)
    n = 50_001
    cols = _random_colors(n, rng)
    ob = C.c_uint32()
    oc = np.zeros((n, 5), np.uint8)
    oracle_lib.psyo_color_compress(cols.ctypes.data, n, oc.ctypes.data, C.byref(ob))
    d_in = torch.from_numpy(cols.view(np.uint8).copy()).cuda()
    d_out = torch.zeros(5 * n, dtype=torch.uint8, device="cuda")
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    _check(lib().psy_color_compress(d_in.data_ptr(), n, d_out.data_ptr(), bad.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy().reshape(n, 5), oc) and int(bad.item()) == ob.value > 0

    recs = rng.integers(0, 256, (n, 5), dtype=np.uint8)
    recs[:, 0] = rng.choice([0, 1, 2, 9], n)
    ocol = np.zeros(n, abi.color_dtype())
    oracle_lib.psyo_color_decompress(recs.ctypes.data, n, ocol.ctypes.data, C.byref(ob))
    d_rec = torch.from_numpy(recs.reshape(-1).copy()).cuda()
    d_col = torch.zeros(16 * n, dtype=torch.uint8, device="cuda")
    bad.zero_()
    _check(lib().psy_color_decompress(d_rec.data_ptr(), n, d_col.data_ptr(), bad.data_ptr(), None))
    torch.cuda.synchronize()
    gcol = d_col.cpu().numpy().view(abi.color_dtype())
    assert np.array_equal(gcol["kind"], ocol["kind"]) and same_floats(gcol["v"], ocol["v"])
    assert int(bad.item()) == ob.value > 0

    sh = np.zeros(n, abi.shader_dtype())
    sh["kind"] = rng.choice([0, 1, 2, 2, 5], n)
    sh["color"] = _random_colors(n, rng)
    sh["roughness"] = rng.uniform(-0.5, 1.5, n).astype(np.float32)
    sh["fresnel"] = cc.random_triples(n, seed=5)[:, 0]
    for stride in (6, 10, 13):
        orec = np.full((n, stride), 0xab, np.uint8)
        oracle_lib.psyo_closure_compress(sh.ctypes.data, n, stride, orec.ctypes.data, C.byref(ob))
        d_sh = torch.from_numpy(sh.view(np.uint8).copy()).cuda()
        d_rec = torch.full((n * stride,), 0xab, dtype=torch.uint8, device="cuda")
        bad.zero_()
        _check(lib().psy_closure_compress(d_sh.data_ptr(), n, stride, d_rec.data_ptr(), bad.data_ptr(), None))
        torch.cuda.synchronize()
        grec = d_rec.cpu().numpy().reshape(n, stride)
        assert np.array_equal(grec, orec) and int(bad.item()) == ob.value > 0, stride
        osh = np.zeros(n, abi.shader_dtype())
        oracle_lib.psyo_closure_decompress(orec.ctypes.data, n, stride, osh.ctypes.data, C.byref(ob))
        d_out = torch.zeros(28 * n, dtype=torch.uint8, device="cuda")
        bad.zero_()
        _check(lib().psy_closure_decompress(d_rec.data_ptr(), n, stride, d_out.data_ptr(), bad.data_ptr(), None))
        torch.cuda.synchronize()
        gsh = d_out.cpu().numpy().view(abi.shader_dtype())
        assert int(bad.item()) == ob.value, stride
        assert np.array_equal(gsh["kind"], osh["kind"]) and np.array_equal(gsh["color"]["kind"], osh["color"]["kind"])
        assert same_floats(gsh["color"]["v"], osh["color"]["v"])
        assert same_floats(gsh["roughness"], osh["roughness"]) and same_floats(gsh["fresnel"], osh["fresnel"])


def test_crate_style_interface():
    """The module-level API reads like the crate's own tests."""
    assert compact.fluv32.encode((1.0, 1.0, 1.0)) == 0x7e0056c3
    assert compact.fluv32.decode_yuv(compact.fluv32.encode((1.0, 1.0, 1.0))) == (1.0, 0x56, 0xc3)
    assert compact.fluv32.decode(0xFFFFFFFF)[1] == compact.fluv32.Y_MAX
    assert compact.unsigned32.encode((float("inf"), 0.0, 0.0)) == 0xFF80001F
    assert compact.unsigned40.encode_64((float("inf"), 0.0, 0.0)) == 0xffe000007f
    assert compact.unsigned40.encode((float("inf"), 0.0, 0.0)) == bytes([0x7f, 0, 0, 0xe0, 0xff])
    assert compact.signed48.encode_64((float("-inf"), 0.0, 0.0)) == 0xFFFC0000003F
    assert compact.signed48.decode_64(0xFFFF_FFFF_FFFF) == (compact.signed48.MIN,) * 3
    assert compact.oct32.decode(compact.oct32.encode_precise((0.0, 0.0, -1.0))) == (0.0, 0.0, -1.0)
    with pytest.raises(ValueError):
        compact.fluv32.encode((float("nan"), 0.0, 0.0))
    with pytest.raises(ValueError):
        compact.unsigned32.encode((0.0, -1.0, 0.0))
    compact.unsigned32.encode((-0.0, -0.0, -0.0))
    assert compact.unsigned32.encode((0.0, -1.0, 0.0), check=False) == 0  # release build: clamps to 0
    batch = compact.signed48.encode(np.ones((4, 2, 3), np.float32))
    assert batch.shape == (4, 2, 6)
    assert np.array_equal(compact.signed48.decode(batch), np.ones((4, 2, 3), np.float32))
    cols = np.zeros(2, abi.color_dtype())
    cols["kind"] = [abi.PSY_COLOR_XYZ, abi.PSY_COLOR_BLACKBODY]
    cols["v"] = [(1.0, 1.0, 1.0), (6500.0, 2.0, 0.0)]
    rec = compact.color_compress(cols)
    assert rec.tolist() == [[0, 0xc3, 0x56, 0x00, 0x7e], [1, 0x64, 0x19, 0x00, 0x40]]
    assert compact.color_decompress(rec)["v"][1].tolist() == [6500.0, 2.0, 0.0]


def test_closure_records_through_the_python_interface(oracle_lib):
    """closure_compress / closure_decompress (the MicropolyBatch record
    layout) equal the oracle's records and round-trip the closures to the
    records' precision."""
    import ctypes as C
    sh = np.zeros(3, abi.shader_dtype())
    sh["kind"] = [abi.PSY_SHADER_LAMBERT, abi.PSY_SHADER_GGX, abi.PSY_SHADER_EMIT]
    sh["color"]["kind"] = [abi.PSY_COLOR_XYZ, abi.PSY_COLOR_BLACKBODY, abi.PSY_COLOR_TEMPERATURE]
    sh["color"]["v"] = [(0.25, 0.5, 0.75), (6500.0, 2.0, 0.0), (3000.0, 0.5, 0.0)]
    sh["roughness"] = [0.0, 0.5, 0.0]
    sh["fresnel"] = [0.0, 0.25, 0.0]
    rec = compact.closure_compress(sh)
    assert rec.shape == (3, 10)
    want = np.zeros((3, 10), np.uint8)
    bad = C.c_uint32()
    assert oracle_lib.psyo_closure_compress(sh.ctypes.data, 3, 10, want.ctypes.data, C.byref(bad)) == 0
    assert np.array_equal(rec, want) and bad.value == 0
    back = compact.closure_decompress(rec)
    assert back["kind"].tolist() == sh["kind"].tolist()
    assert back["color"]["kind"].tolist() == sh["color"]["kind"].tolist()
    assert back[1]["roughness"] == np.float32(32767) * np.float32(1.0 / 65535.0)
    assert back[1]["fresnel"] == np.float32(16383) * np.float32(1.0 / 65535.0)
    assert back[1]["color"]["v"].tolist() == [6500.0, 2.0, 0.0]
    assert np.allclose(back[0]["color"]["v"], sh[0]["color"]["v"], rtol=0.02)
    with pytest.raises(ValueError):
        compact.closure_compress(sh, stride=6)  # the GGX record does not fit
