"""The `compact` crate's encodings (sub_crates/compact), computed on the GPU
through the C ABI (psy_compact_*, psy_fluv32_decode_yuv), plus the colour and
closure byte formats built on them (psy_color_*, psy_closure_*).  The module
layout and function names follow the crate:

    fluv32.encode(xyz) -> u32        fluv32.decode(u32) -> (x, y, z)
    fluv32.decode_yuv(u32) -> (y, u, v)
    oct32.encode(v) / oct32.encode_precise(v) -> u32, oct32.decode(u32)
    unsigned32.encode(fs) -> u32     unsigned32.decode(u32)
    unsigned40.encode(fs) -> 5 bytes unsigned40.decode(5 bytes)
    signed48.encode(fs) -> 6 bytes   signed48.decode(6 bytes)

Each call takes one triple (a tuple: the crate's signature) or an array of
shape (..., 3) (a batch: one kernel launch) and returns one code or an array
of codes -- uint32 for the 4-byte formats, uint8 (..., 5) / (..., 6) for
unsigned40 / signed48 (the crate's [u8; 5] / [u8; 6]).  Encoding a value
outside the format's domain (a NaN or negative component for fluv32,
unsigned32 and unsigned40; a NaN for signed48) raises ValueError, as the
crate's debug assertions panic; check=False returns the release build's
code instead.

The CUDA library is required; there is no CPU fallback.
"""
import numpy as np

from . import abi
from .gpu import _check, lib


def element_size(fmt):
    """Bytes per code of a PSY_COMPACT_* format (psy_compact_element_size)."""
    import ctypes as C
    b = C.c_uint32()
    _check(lib().psy_compact_element_size(fmt, C.byref(b)))
    return b.value


def encode_device(fmt, d_xyz_ptr, n, d_out_ptr, d_invalid_ptr=None, stream=None):
    """psy_compact_encode on device buffers (asynchronous on `stream`)."""
    _check(lib().psy_compact_encode(fmt, d_xyz_ptr, n, d_out_ptr, d_invalid_ptr, stream))


def decode_device(fmt, d_in_ptr, n, d_xyz_ptr, stream=None):
    """psy_compact_decode on device buffers (asynchronous on `stream`)."""
    _check(lib().psy_compact_decode(fmt, d_in_ptr, n, d_xyz_ptr, stream))


def _to_device(a):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a).reshape(-1).view(np.uint8).copy())
    return t.cuda() if t.numel() else torch.empty(1, dtype=torch.uint8, device="cuda")


def _from_device(t, nbytes):
    import torch
    torch.cuda.synchronize()
    return t[:nbytes].cpu().numpy() if nbytes else np.zeros(0, np.uint8)


def _invalid_counter():
    import torch
    return torch.zeros(1, dtype=torch.int32, device="cuda")


def _raise_invalid(bad, what):
    if bad:
        raise ValueError("%s: %d input(s) outside the format's domain" % (what, bad))


def encode(fmt, xyz, check=True):
    """Batch encode: xyz (..., 3) float32 -> codes; see the module docstring."""
    import torch
    a = np.ascontiguousarray(np.asarray(xyz, dtype=np.float32))
    if a.ndim == 0 or a.shape[-1] != 3:
        raise ValueError("encode: the last axis must hold the three components")
    lead = a.shape[:-1]
    n = int(np.prod(lead, dtype=np.int64))
    size = element_size(fmt)
    d_in = _to_device(a)
    d_out = torch.empty(max(1, n * size), dtype=torch.uint8, device="cuda")
    bad = _invalid_counter()
    encode_device(fmt, d_in.data_ptr(), n, d_out.data_ptr(), bad.data_ptr())
    raw = _from_device(d_out, n * size)
    if check:
        _raise_invalid(int(bad.item()), "encode")
    if size == 4:
        codes = raw.view("<u4").reshape(lead)
        return int(codes) if lead == () else codes
    codes = raw.reshape(lead + (size,))
    return bytes(codes) if lead == () else codes


def decode(fmt, codes):
    """Batch decode: codes -> (..., 3) float32 (a tuple for one code)."""
    import torch
    size = element_size(fmt)
    if size == 4:
        c = np.asarray(codes, dtype=np.uint64).astype(np.uint32)  # keeps a scalar's shape ()
        lead = c.shape
    else:
        if isinstance(codes, (bytes, bytearray)):
            codes = np.frombuffer(bytes(codes), dtype=np.uint8)
        c = np.asarray(codes, dtype=np.uint8)
        if c.ndim == 0 or c.shape[-1] != size:
            raise ValueError("decode: the last axis must hold %d bytes" % size)
        lead = c.shape[:-1]
    n = int(np.prod(lead, dtype=np.int64))
    d_in = _to_device(c)
    d_out = torch.empty(max(1, 3 * n), dtype=torch.float32, device="cuda")
    decode_device(fmt, d_in.data_ptr(), n, d_out.data_ptr())
    torch.cuda.synchronize()
    out = d_out[:3 * n].cpu().numpy().reshape(lead + (3,))
    return tuple(float(v) for v in out) if lead == () else out


class _Format:
    def __init__(self, fmt):
        self._fmt = fmt

    def encode(self, floats, check=True):
        return encode(self._fmt, floats, check)

    def decode(self, code):
        return decode(self._fmt, code)


class _Fluv32(_Format):
    """fluv::fluv32 (sub_crates/compact/src/fluv/fluv32.rs)."""
    U_SCALE = float(np.float32(817.0) / np.float32(2.0))
    V_SCALE = float(np.float32(1235.0) / np.float32(3.0))
    Y_MAX = float(np.float32((1 << 65) - (1 << 55)))
    Y_MIN = float(np.float32(1.0) / np.float32(float(1 << 62)))
    Y_EPSILON = 1.0 / 512.0

    def decode_yuv(self, code):
        """(Y, u', v') of each code: Y as float32, the chroma as the raw bytes."""
        import torch
        c = np.asarray(code, dtype=np.uint64).astype(np.uint32)  # keeps a scalar's shape ()
        n = c.size
        d_in = _to_device(c)
        d_out = torch.empty(max(1, 8 * n), dtype=torch.uint8, device="cuda")
        _check(lib().psy_fluv32_decode_yuv(d_in.data_ptr(), n, d_out.data_ptr(), None))
        r = _from_device(d_out, 8 * n).view(abi.yuv_dtype()).reshape(c.shape)
        if c.shape == ():
            return float(r["y"]), int(r["u"]), int(r["v"])
        return r["y"], r["u"], r["v"]


class _Oct32(_Format):
    """unit_vec::oct32 (sub_crates/compact/src/unit_vec/oct32.rs)."""

    def encode_precise(self, vec):
        return encode(abi.PSY_COMPACT_OCT32_PRECISE, vec, check=False)


class _SharedExp(_Format):
    """shared_exp::{unsigned32, unsigned40, signed48}; encode_64 / decode_64
    give the crate's u64 workhorse form of the byte-array codes."""

    def __init__(self, fmt, max_value, min_value, epsilon, min_positive=None):
        super().__init__(fmt)
        self.MAX, self.MIN, self.EPSILON = max_value, min_value, epsilon
        if min_positive is not None:
            self.MIN_POSITIVE = min_positive

    def encode_64(self, floats, check=True):
        c = self.encode(floats, check)
        return c if isinstance(c, int) else int.from_bytes(c, "little")

    def decode_64(self, n):
        size = element_size(self._fmt)
        return self.decode(n if size == 4 else (int(n) & ((1 << (8 * size)) - 1)).to_bytes(size, "little"))


fluv32 = _Fluv32(abi.PSY_COMPACT_FLUV32)
oct32 = _Oct32(abi.PSY_COMPACT_OCT32)
unsigned32 = _SharedExp(abi.PSY_COMPACT_UNSIGNED32, float(np.float32((1 << 21) - (1 << 12))), 2.0 ** -19, 1.0 / 256)
unsigned40 = _SharedExp(abi.PSY_COMPACT_UNSIGNED40, float(np.float32((1 << 96) - (1 << 85))), 2.0 ** -42, 1.0 / 1024)
signed48 = _SharedExp(abi.PSY_COMPACT_SIGNED48, float(np.float32((1 << 38) - (1 << 25))),
                      -float(np.float32((1 << 38) - (1 << 25))), 1.0 / 4096, min_positive=2.0 ** -38)


def color_compress(colors, check=True):
    """Color::write_compressed for an array of PsyColor records
    (abi.color_dtype()): (n, 5) uint8."""
    import torch
    c = np.ascontiguousarray(np.asarray(colors, dtype=abi.color_dtype()).reshape(-1))
    n = c.size
    d_in = _to_device(c)
    d_out = torch.empty(max(1, 5 * n), dtype=torch.uint8, device="cuda")
    bad = _invalid_counter()
    _check(lib().psy_color_compress(d_in.data_ptr(), n, d_out.data_ptr(), bad.data_ptr(), None))
    raw = _from_device(d_out, 5 * n)
    if check:
        _raise_invalid(int(bad.item()), "color compress")
    return raw.reshape(n, 5)


def color_decompress(data):
    """Color::from_compressed for (n, 5) uint8 records: PsyColor records."""
    import torch
    d = np.ascontiguousarray(np.asarray(data, dtype=np.uint8).reshape(-1, 5))
    n = d.shape[0]
    d_in = _to_device(d)
    d_out = torch.empty(max(1, 16 * n), dtype=torch.uint8, device="cuda")
    bad = _invalid_counter()
    _check(lib().psy_color_decompress(d_in.data_ptr(), n, d_out.data_ptr(), bad.data_ptr(), None))
    raw = _from_device(d_out, 16 * n)
    _raise_invalid(int(bad.item()), "color decompress")
    return raw.view(abi.color_dtype())


def closure_compress(closures, stride=None, check=True):
    """SurfaceClosure::write_compressed for PsyShaderDesc records
    (abi.shader_dtype()) at a fixed stride (default: the largest record,
    10 bytes with a GGX closure, else 6): (n, stride) uint8, bytes past a
    record's end zero."""
    import torch
    s = np.ascontiguousarray(np.asarray(closures, dtype=abi.shader_dtype()).reshape(-1))
    n = s.size
    if stride is None:
        stride = 10 if np.any(s["kind"] == abi.PSY_SHADER_GGX) else 6
    d_in = _to_device(s)
    d_out = torch.zeros(max(1, stride * n), dtype=torch.uint8, device="cuda")
    bad = _invalid_counter()
    _check(lib().psy_closure_compress(d_in.data_ptr(), n, stride, d_out.data_ptr(), bad.data_ptr(), None))
    raw = _from_device(d_out, stride * n)
    if check:
        _raise_invalid(int(bad.item()), "closure compress")
    return raw.reshape(n, stride)


def closure_decompress(data):
    """SurfaceClosure::from_compressed for (n, stride) uint8 records."""
    import torch
    d = np.ascontiguousarray(np.asarray(data, dtype=np.uint8))
    n, stride = d.shape
    d_in = _to_device(d)
    d_out = torch.empty(max(1, 28 * n), dtype=torch.uint8, device="cuda")
    bad = _invalid_counter()
    _check(lib().psy_closure_decompress(d_in.data_ptr(), n, stride, d_out.data_ptr(), bad.data_ptr(), None))
    raw = _from_device(d_out, 28 * n)
    _raise_invalid(int(bad.item()), "closure decompress")
    return raw.view(abi.shader_dtype())
