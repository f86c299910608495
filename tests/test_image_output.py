"""Image output: the PNG writer (CPU) and the GPU XYZ -> sRGB8 conversion
against the oracle's restatement of Image::write_png (src/image.rs:138-164).
The conversion differs only where CUDA's powf and the host's pow round the
gamma curve differently next to a quantisation step: at most 1 in a
channel, on at most 0.1% of channel values (stated bar)."""
import ctypes as C

import numpy as np
import pytest

from psychopath_gb300 import image


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    rgba = rng.integers(0, 256, size=(7, 13, 4), dtype=np.uint8)
    data = image.png_bytes(rgba)
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    assert np.array_equal(image.read_png_rgba(data), rgba)
    p = tmp_path / "x.png"
    image.write_png(str(p), rgba)
    assert np.array_equal(image.read_png_rgba(p.read_bytes()), rgba)


def _oracle_srgb8(oracle_lib, xyz):
    h, w = xyz.shape[:2]
    out = np.zeros((h, w, 4), dtype=np.uint8)
    x = np.ascontiguousarray(xyz, dtype=np.float32)
    oracle_lib.psyo_xyz_to_srgb8(x.ctypes.data_as(C.POINTER(C.c_float)), w, h, out.ctypes.data)
    return out


def test_oracle_conversion_known_values(oracle_lib):
    # XYZ (1, 1, 1) is equal-energy white: rec709_e (1, 1, 1) up to the
    # 10-decimal rounding of the matrix, which leaves each channel just below
    # 1 -- 254.99..., truncated to 254 as the reference quantises; black
    # stays black; the last image row becomes the first PNG row
    xyz = np.zeros((2, 1, 3), dtype=np.float32)
    xyz[1, 0] = 1.0  # bottom row white
    out = _oracle_srgb8(oracle_lib, xyz)
    assert out[0, 0].tolist() == [254, 254, 254, 255] and out[1, 0].tolist() == [0, 0, 0, 255]
    # a mid grey: Y = 0.2 -> gamma(0.2) = 0.4845..., x 255 = 123.5... -> 123
    xyz = np.full((1, 1, 3), 0.2, dtype=np.float32)
    assert _oracle_srgb8(oracle_lib, xyz)[0, 0, :3].tolist() == [123, 123, 123]


@pytest.mark.gpu
def test_gpu_conversion_matches_oracle(gpu_lib, oracle_lib):
    rng = np.random.default_rng(5)
    xyz = (rng.random((64, 96, 3)) ** 2 * 1.3).astype(np.float32)
    xyz[0, :4] = [[0, 0, 0], [np.nan, 0, 0], [5, 5, 5], [-1, 0.2, 0.1]]
    got = image.xyz_to_srgb8(xyz)
    ref = _oracle_srgb8(oracle_lib, xyz)
    d = np.abs(got.astype(int) - ref.astype(int))
    assert d.max() <= 1
    assert (d > 0).mean() <= 1e-3


def test_exr_round_trip_and_layout(tmp_path):
    rng = np.random.default_rng(2)
    xyz = (rng.random((5, 9, 3)) * 4.0).astype(np.float32)
    data = image.exr_bytes(xyz)
    # magic, version 2 (single-part scanline), then the header attributes
    assert data[:8] == bytes([0x76, 0x2F, 0x31, 0x01, 2, 0, 0, 0])
    for name in (b"channels\0chlist", b"compression\0compression", b"dataWindow\0box2i", b"displayWindow\0box2i",
                 b"lineOrder\0lineOrder", b"pixelAspectRatio\0float", b"screenWindowCenter\0v2f",
                 b"screenWindowWidth\0float"):
        assert name in data
    got = image.read_exr_rgb(data)
    assert np.array_equal(got, image.xyz_to_rec709_e(xyz).astype(np.float16))
    image.write_exr(str(tmp_path / "x.exr"), xyz)


def test_xyz_to_rec709_e_matches_oracle_matrix(oracle_lib):
    """The host matrix equals the oracle's (both restate the color crate's
    generator): XYZ (1, 1, 1) maps to its rec709_e white, and the conversion
    inverts rec709_e_to_xyz to f32 precision."""
    from psychopath_gb300 import scenes
    white = image.xyz_to_rec709_e(np.ones(3, dtype=np.float32))
    assert np.allclose(white, 1.0, atol=1e-6)
    rgb = np.array([0.2, 0.5, 0.9], dtype=np.float32)
    back = image.xyz_to_rec709_e(scenes.rec709_e_to_xyz(rgb))
    assert np.allclose(back, rgb, atol=1e-6)
    # PNG path on the oracle: same matrix -> the oracle's srgb8 of a pixel
    # equals the host conversion followed by the same gamma and quantisation
    xyz = np.array([[[0.3, 0.4, 0.5]]], dtype=np.float32)
    out = _oracle_srgb8(oracle_lib, xyz)[0, 0, :3]
    lin = image.xyz_to_rec709_e(xyz)[0, 0]
    g = np.where(lin < np.float32(0.0031308), lin * np.float32(12.92),
                 np.float32(1.055) * np.power(lin, np.float32(1.0) / np.float32(2.4)) - np.float32(0.055))
    q = (np.minimum(np.float32(1), np.maximum(np.float32(0), g)) * np.float32(255)).astype(np.uint8)
    assert np.abs(q.astype(int) - out.astype(int)).max() <= 1
