"""Serialized bucket output for PsychoBlend (the reference's
`--serialized_output` mode), driven by the GPU bucket render.

The reference's renderer splits the image into square buckets of about
`max_samples_per_bucket / spp` pixels (src/renderer.rs:138-147), queues them
in Hilbert-curve order (src/renderer.rs:149-180, src/hilbert.rs:47-63) and,
after each bucket, prints to stdout (src/renderer.rs:312-343):

    DIV
    <percentage of pixels done, two decimals>%
    <min x> <min y> <max x> <max y>
    <base64 of the bucket's pixels as f32 RGBA, linear rec709 (equal-energy
     white), alpha 1, scanline order (src/image.rs:229-256)>
    BUCKET_END
    DIV

Here every bucket is rendered on the GPU by psy_render_bucket in the same
order and written in the same format, so the Blender add-on's reader
(psychoblend/render.py) can consume it unchanged.
"""
import base64
import math
import sys

import numpy as np

from .image import xyz_to_rec709_e

HILBERT_N = 1 << 16


def _hil_rot(n, rx, ry, x, y):
    if ry == 0:
        if rx == 1:
            x = (n - 1 - x) & 0xFFFFFFFF
            y = (n - 1 - y) & 0xFFFFFFFF
        x, y = y, x
    return x, y


def hilbert_d2xy(d):
    """Point of the 2^16 x 2^16 Hilbert curve at distance d (src/hilbert.rs:47-63)."""
    x, y, s, t = 0, 0, 1, d
    while s < HILBERT_N:
        rx = 1 & (t >> 1)
        ry = 1 & (t ^ rx)
        x, y = _hil_rot(s, rx, ry, x, y)
        x += s * rx
        y += s * ry
        t >>= 2
        s <<= 1
    return x, y


def hilbert_xy2d(x, y):
    """Distance along the curve of point (x, y) (src/hilbert.rs:25-45)."""
    d, s = 0, HILBERT_N >> 1
    while s > 0:
        rx = 1 if (x & s) else 0
        ry = 1 if (y & s) else 0
        d += s * s * ((3 * rx) ^ ry)
        x, y = _hil_rot(s, rx, ry, x, y)
        s >>= 1
    return d


def bucket_size(spp, max_samples_per_bucket=4096):
    """Side of the square buckets (src/renderer.rs:138-147): the integer part
    of sqrt(max_samples_per_bucket / spp) computed in f64, at least 1."""
    target = float(max_samples_per_bucket) / float(spp)
    side = math.sqrt(target)
    return 1 if side < 1.0 else int(side)


def bucket_jobs(width, height, spp, max_samples_per_bucket=4096, start=(0, 0)):
    """Buckets (x, y, w, h) in the reference's queue order: Hilbert order
    over a power-of-two square of bucket cells, cells outside the image
    dropped, edge buckets clipped (src/renderer.rs:149-180)."""
    bw = bh = bucket_size(spp, max_samples_per_bucket)
    nx, ny = width // bw + 1, height // bh + 1
    larger = max(nx, ny)
    pow2 = 1 << (larger - 1).bit_length() if larger > 1 else 1
    jobs = []
    for d in range(pow2 * pow2):
        bx, by = hilbert_d2xy(d)
        x, y = bx * bw, by * bh
        w = min(bw, width - x) if width >= x else bw
        h = min(bh, height - y) if height >= y else bh
        if x < width and y < height and w > 0 and h > 0:
            jobs.append((start[0] + x, start[1] + y, w, h))
    return jobs


def bucket_rgba_base64(xyz_bucket):
    """Bucket pixels (h, w, 3) XYZ -> base64 of f32 RGBA in linear rec709
    (equal-energy white), alpha 1.0, scanline order (Bucket::rgba_base64)."""
    rgb = xyz_to_rec709_e(np.asarray(xyz_bucket, dtype=np.float32))
    h, w = rgb.shape[:2]
    rgba = np.ones((h, w, 4), dtype="<f4")
    rgba[..., :3] = rgb
    return base64.b64encode(rgba.tobytes()).decode("ascii")


def bucket_record(xyz_bucket, x, y, pixels_done, total_pixels):
    """The lines printed for one finished bucket (src/renderer.rs:320-342)."""
    h, w = xyz_bucket.shape[:2]
    pct = "%.2f%%" % (pixels_done / total_pixels * 100.0)
    return "DIV\n%s\n%d %d %d %d\n%s\nBUCKET_END\nDIV\n" % (pct, x, y, x + w, y + h,
                                                         bucket_rgba_base64(xyz_bucket))


def parse_records(text, width, height):
    """Reassembles the linear rec709 RGBA image (height, width, 4) from a
    serialized stream, as the add-on does; returns (image, percentages)."""
    img = np.zeros((height, width, 4), dtype=np.float32)
    pcts = []
    lines = text.split("\n")
    i = 0
    while i < len(lines):
        if lines[i] == "DIV" and i + 4 < len(lines) and lines[i + 4] == "BUCKET_END":
            pcts.append(lines[i + 1])
            x0, y0, x1, y1 = (int(v) for v in lines[i + 2].split())
            data = np.frombuffer(base64.b64decode(lines[i + 3]), dtype="<f4").reshape(y1 - y0, x1 - x0, 4)
            img[y0:y1, x0:x1] = data
            i += 6
        else:
            i += 1
    return img, pcts


def render_serialized(renderer, out=None, max_samples_per_bucket=4096, spp=None, seed=None):
    """Renders the scene bucket by bucket on the GPU (psy_render_bucket) in the
    reference's bucket order and writes the serialized records to `out`
    (default: stdout) after each bucket.  Returns the XYZ image."""
    out = out or sys.stdout
    sc = renderer.scene
    W, H = sc.width, sc.height
    spp = spp if spp is not None else sc.spp
    img = np.zeros((H, W, 3), dtype=np.float32)
    done = 0
    for (x, y, w, h) in bucket_jobs(W, H, spp, max_samples_per_bucket):
        xyz, _ = renderer.render_bucket(x, y, w, h, spp=spp, seed=seed)
        img[y:y + h, x:x + w] = xyz
        done += w * h
        out.write(bucket_record(xyz, x, y, done, W * H))
        out.flush()
    return img
