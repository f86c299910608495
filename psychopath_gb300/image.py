"""Image output of a render: the XYZ image to sRGB RGBA8 on the GPU
(psy_xyz_to_srgb8, the conversion of the reference's Image::write_png,
src/image.rs:138-164) and a PNG file writer.

The PNG writer emits the format's standard chunks (signature, IHDR, IDAT,
IEND; RGBA, 8 bits per channel, no interlacing, filter type 0 on every row)
with the zlib stream from Python's standard library.
"""
import ctypes as C
import struct
import zlib

import numpy as np

from . import gpu


def xyz_to_srgb8_device(d_xyz_ptr, width, height, d_rgba_ptr, stream=None):
    """psy_xyz_to_srgb8 on device buffers (width*height*3 floats in,
    width*height*4 bytes out, rows flipped for PNG)."""
    gpu._check(gpu.lib().psy_xyz_to_srgb8(C.c_void_p(d_xyz_ptr), width, height, C.c_void_p(d_rgba_ptr), stream))


def xyz_to_srgb8(xyz):
    """Host XYZ image (height, width, 3) float32 -> (height, width, 4) uint8
    through the GPU conversion."""
    import torch
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    h, w = xyz.shape[:2]
    d_in = torch.from_numpy(xyz.reshape(-1)).cuda()
    d_out = torch.empty(h * w * 4, dtype=torch.uint8, device="cuda")
    xyz_to_srgb8_device(d_in.data_ptr(), w, h, d_out.data_ptr())
    torch.cuda.synchronize()
    return d_out.cpu().numpy().reshape(h, w, 4)


def png_bytes(rgba):
    """(height, width, 4) uint8 -> PNG file contents."""
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = rgba.shape[:2]
    raw = np.zeros((h, 1 + 4 * w), dtype=np.uint8)  # filter byte 0, then the row
    raw[:, 1:] = rgba.reshape(h, 4 * w)

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    ihdr = struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)  # 8-bit RGBA
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", ihdr) + chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)) +
            chunk(b"IEND", b""))


def write_png(path, rgba):
    with open(path, "wb") as f:
        f.write(png_bytes(rgba))


def read_png_rgba(data):
    """Decode what png_bytes writes (8-bit RGBA, filter 0): for checks."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, w, h, idat = 8, 0, 0, b""
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(tag + body) & 0xFFFFFFFF, "bad CRC in %r" % tag
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 6
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + 4 * w)
    assert (raw[:, 0] == 0).all()
    return raw[:, 1:].reshape(h, w, 4)
