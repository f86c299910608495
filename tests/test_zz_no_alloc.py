"""psy_render_bucket_noalloc: the bucket render for hosts that cannot call
cudaMalloc after start-up (their device memory is reserved up front, or they
must keep a fixed footprint).  Called through the C ABI, its output must
equal the allocating psy_render_bucket's output exactly, on two calls in a
row (the calls share one static scratch array).  This file is collected last
so a failure here cannot hide the results of the other tests."""
import ctypes as C

import numpy as np
import pytest

from psychopath_gb300 import abi, gpu, scenes

pytestmark = pytest.mark.gpu


def _scene():
    return scenes.cornell_box(64, 64, 16, max_bounces=4)


def test_noalloc_matches_allocating_bucket_render(gpu_lib):
    torch = pytest.importorskip("torch")
    sd = _scene()
    g = gpu.Scene(sd)
    r = gpu.Renderer(g)
    x, y, w, h = 16, 8, 32, 24  # 32*24*16 = 12,288 samples
    ref, _ = r.render_bucket(x, y, w, h)
    out = torch.zeros(w * h * 3, dtype=torch.float32, device="cuda")
    for call in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        r.render_bucket_noalloc(x, y, w, h, out.data_ptr())
        got = out.cpu().numpy().reshape(h, w, 3)
        assert np.isfinite(got).all()
        assert np.array_equal(got, ref), "call %d differs from psy_render_bucket" % call
    g.close()


def test_noalloc_rejects_oversize_bucket(gpu_lib):
    torch = pytest.importorskip("torch")
    sd = _scene()
    g = gpu.Scene(sd)
    out = torch.zeros(64 * 64 * 3, dtype=torch.float32, device="cuda")
    b = abi.PsyBucket(0, 0, 64, 64)
    spp = abi.PSY_NOALLOC_MAX_SAMPLES // (64 * 64) + 1
    rc = gpu_lib.psy_render_bucket_noalloc(g.h, C.byref(b), spp, 0, C.c_void_p(out.data_ptr()), None)
    assert rc == abi.PSY_E_INVALID
    assert b"no-allocation" in gpu_lib.psy_last_error()
    g.close()
