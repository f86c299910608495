"""Serialized bucket output (the reference's --serialized_output mode read by
PsychoBlend): bucket size and Hilbert queue order as src/renderer.rs:138-180,
the record format of src/renderer.rs:312-343 and Bucket::rgba_base64
(src/image.rs:229-256).  The bucket order is checked against the CPU
oracle's bucket scheduler; the GPU test reassembles a serialized render."""
import base64
import io

import numpy as np
import pytest

from oracle.runner import OracleScene
from psychopath_gb300 import blender, image

from . import scene_cases as sc


def test_hilbert_reversible():
    # src/hilbert.rs:65-77: d = 54 round-trips
    x, y = blender.hilbert_d2xy(54)
    assert blender.hilbert_xy2d(x, y) == 54
    for d in range(4096):
        assert blender.hilbert_xy2d(*blender.hilbert_d2xy(d)) == d
    # the curve starts at the origin and moves one cell per step
    pts = [blender.hilbert_d2xy(d) for d in range(256)]
    assert pts[0] == (0, 0)
    assert all(abs(a[0] - b[0]) + abs(a[1] - b[1]) == 1 for a, b in zip(pts, pts[1:]))


@pytest.mark.parametrize("w,h,spp", [(32, 32, 64), (37, 21, 16), (1920, 1080, 64), (5, 3, 5000)])
def test_buckets_partition_the_image(w, h, spp):
    jobs = blender.bucket_jobs(w, h, spp)
    side = blender.bucket_size(spp)
    assert side == max(1, int((4096.0 / spp) ** 0.5))
    cover = np.zeros((h, w), dtype=np.int32)
    for x, y, bw, bh in jobs:
        assert 0 < bw <= side and 0 < bh <= side
        cover[y:y + bh, x:x + bw] += 1
    assert (cover == 1).all()


def test_bucket_order_matches_oracle_scheduler(oracle_lib):
    s = sc.cornell(32, 32, 64, 2)  # bucket side 8: a 4x4 grid queued on an 8x8 Hilbert square
    o = OracleScene(s)
    jobs = blender.bucket_jobs(32, 32, 64)
    for k in (1, 3, 6, 11):
        img, _ = o.render(threads=2, max_buckets=k)
        rendered = np.abs(img).sum(axis=2) > 0
        want = np.zeros((32, 32), dtype=bool)
        for x, y, bw, bh in jobs[:k]:
            want[y:y + bh, x:x + bw] = True
        assert not (rendered & ~want).any(), k
        assert rendered[want].mean() > 0.95, k


def test_record_format():
    rng = np.random.default_rng(3)
    xyz = rng.uniform(0, 2, (3, 4, 3)).astype(np.float32)
    rec = blender.bucket_record(xyz, 8, 16, 24, 96)
    lines = rec.split("\n")
    assert lines[0] == "DIV" and lines[1] == "25.00%" and lines[2] == "8 16 12 19"
    assert lines[4] == "BUCKET_END" and lines[5] == "DIV" and lines[6] == ""
    data = np.frombuffer(base64.b64decode(lines[3]), dtype="<f4").reshape(3, 4, 4)
    assert np.array_equal(data[..., :3], image.xyz_to_rec709_e(xyz))
    assert (data[..., 3] == 1.0).all()
    img, pcts = blender.parse_records(rec, 20, 20)
    assert pcts == ["25.00%"]
    assert np.array_equal(img[16:19, 8:12], data)


@pytest.mark.gpu
def test_serialized_gpu_render_reassembles_image(gpu_lib):
    from psychopath_gb300 import gpu
    s = sc.cornell(40, 24, 16, 2)
    g = gpu.Scene(s)
    r = gpu.Renderer(g)
    full, _ = r.render()
    buf = io.StringIO()
    img = blender.render_serialized(r, out=buf)
    assert np.array_equal(img, full)
    rgba, pcts = blender.parse_records(buf.getvalue(), 40, 24)
    assert pcts[-1] == "100.00%" and len(pcts) == len(blender.bucket_jobs(40, 24, 16))
    assert np.array_equal(rgba[..., :3], image.xyz_to_rec709_e(full))
    g.close()
