"""Image output of a render: the XYZ image to sRGB RGBA8 on the GPU
(psy_xyz_to_srgb8, the conversion of the reference's Image::write_png,
src/image.rs:138-164) and a PNG file writer; and linear rec709 half-float
OpenEXR output (Image::write_exr, src/image.rs:166-196).

The PNG writer emits the format's standard chunks (signature, IHDR, IDAT,
IEND; RGBA, 8 bits per channel, no interlacing, filter type 0 on every row)
with the zlib stream from Python's standard library.  The EXR writer emits
a single-part scanline file with the required header attributes, HALF
channels B, G, R and no compression (the reference asks OpenEXR for PIZ;
pixel values are the same, only the file is larger).
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


# ---------------------------------------------------------------- OpenEXR
def _xyz_to_rec709_e_matrix():
    """The color crate's generated xyz_to_rec709_e constants (inverse of the
    equal-energy rec709 matrix by Gauss-Jordan elimination in f64, printed
    with 10 decimals), as f32."""
    r, g, b, w = (0.640, 0.330), (0.300, 0.600), (0.150, 0.060), (1.0 / 3.0, 1.0 / 3.0)
    Y = 1.0
    X = w[0] * Y / w[1]
    Z = (1.0 - w[0] - w[1]) * Y / w[1]
    d = r[0] * (b[1] - g[1]) + b[0] * (g[1] - r[1]) + g[0] * (r[1] - b[1])
    sr = (X * (b[1] - g[1]) - g[0] * (Y * (b[1] - 1.0) + b[1] * (X + Z)) + b[0] * (Y * (g[1] - 1.0) + g[1] * (X + Z))) / d
    sg = (X * (r[1] - b[1]) + r[0] * (Y * (b[1] - 1.0) + b[1] * (X + Z)) - b[0] * (Y * (r[1] - 1.0) + r[1] * (X + Z))) / d
    sb = (X * (g[1] - r[1]) - r[0] * (Y * (g[1] - 1.0) + g[1] * (X + Z)) + g[0] * (Y * (r[1] - 1.0) + r[1] * (X + Z))) / d
    t = [[sr * r[0], sg * g[0], sb * b[0]], [sr * r[1], sg * g[1], sb * b[1]],
         [sr * (1.0 - r[0] - r[1]), sg * (1.0 - g[0] - g[1]), sb * (1.0 - b[0] - b[1])]]
    inv = [[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]
    for i in range(2):  # forward elimination; pivot = first row with the largest |value|
        p, size = i, abs(t[i][i])
        for j in range(i + 1, 3):
            if abs(t[j][i]) > size:
                p, size = j, abs(t[j][i])
        if p != i:
            t[i], t[p] = t[p], t[i]
            inv[i], inv[p] = inv[p], inv[i]
        for j in range(i + 1, 3):
            f = t[j][i] / t[i][i]
            for k in range(3):
                t[j][k] -= f * t[i][k]
                inv[j][k] -= f * inv[i][k]
    for i in (2, 1, 0):  # back substitution
        f = t[i][i]
        for k in range(3):
            t[i][k] /= f
            inv[i][k] /= f
        for j in range(i):
            g2 = t[j][i]
            for k in range(3):
                t[j][k] -= g2 * t[i][k]
                inv[j][k] -= g2 * inv[i][k]
    return np.array([[float("%.10f" % inv[i][k]) for k in range(3)] for i in range(3)], dtype=np.float32)


def xyz_to_rec709_e(xyz):
    """(..., 3) float32 XYZ -> linear rec709 (equal-energy white) in f32 with
    the generated code's order: (x*m0 + y*m1) + z*m2."""
    m = _xyz_to_rec709_e_matrix()
    x = np.asarray(xyz, dtype=np.float32)
    out = np.empty_like(x)
    for i in range(3):
        out[..., i] = (x[..., 0] * m[i, 0] + x[..., 1] * m[i, 1]) + x[..., 2] * m[i, 2]
    return out


def _attr(name, typ, data):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(data)) + data


def exr_bytes(xyz):
    """(height, width, 3) XYZ -> OpenEXR file contents: rec709 (equal-energy
    white) as HALF channels R, G, B, row 0 at the top, as
    Image::write_exr stores it (no vertical flip)."""
    rgb = xyz_to_rec709_e(xyz).astype(np.float16)  # round to nearest even, as f16::from_f32
    h, w = rgb.shape[:2]
    chans = b""
    for c in (b"B", b"G", b"R"):  # channel list in alphabetical order
        chans += c + b"\0" + struct.pack("<iB3xii", 1, 0, 1, 1)  # HALF, not linear, sampling 1 x 1
    chans += b"\0"
    box = struct.pack("<iiii", 0, 0, w - 1, h - 1)
    header = (_attr("channels", "chlist", chans) + _attr("compression", "compression", b"\0") +
              _attr("dataWindow", "box2i", box) + _attr("displayWindow", "box2i", box) +
              _attr("lineOrder", "lineOrder", b"\0") + _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) +
              _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)) +
              _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0")
    head = struct.pack("<ii", 20000630, 2) + header
    line = 2 * w * 3
    table_start = len(head)
    first = table_start + 8 * h
    offsets = struct.pack("<%dQ" % h, *[first + y * (8 + line) for y in range(h)])
    blocks = []
    for y in range(h):
        row = rgb[y]
        data = row[:, 2].tobytes() + row[:, 1].tobytes() + row[:, 0].tobytes()  # B, G, R
        blocks.append(struct.pack("<ii", y, len(data)) + data)
    return head + offsets + b"".join(blocks)


def write_exr(path, xyz):
    with open(path, "wb") as f:
        f.write(exr_bytes(xyz))


def read_exr_rgb(data):
    """Decode what exr_bytes writes (single part, scanline, no compression,
    HALF B/G/R): (height, width, 3) float16 R, G, B.  For checks."""
    magic, version = struct.unpack("<ii", data[:8])
    assert magic == 20000630 and (version & 0xFF) == 2
    pos, attrs = 8, {}
    while data[pos] != 0:
        n_end = data.index(b"\0", pos)
        name = data[pos:n_end].decode()
        t_end = data.index(b"\0", n_end + 1)
        typ = data[n_end + 1:t_end].decode()
        size = struct.unpack("<i", data[t_end + 1:t_end + 5])[0]
        attrs[name] = (typ, data[t_end + 5:t_end + 5 + size])
        pos = t_end + 5 + size
    pos += 1
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    assert attrs["compression"][1] == b"\0"
    offs = struct.unpack("<%dQ" % h, data[pos:pos + 8 * h])
    out = np.zeros((h, w, 3), dtype=np.float16)
    for y in range(h):
        o = offs[y]
        yy, size = struct.unpack("<ii", data[o:o + 8])
        px = np.frombuffer(data[o + 8:o + 8 + size], dtype=np.float16).reshape(3, w)
        out[yy, :, 2], out[yy, :, 1], out[yy, :, 0] = px[0], px[1], px[2]
    return out
