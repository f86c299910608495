"""Render server (psy_server_*, psy_submit / psy_poll / psy_wait /
psy_cancel): requests of different scenes, resolutions, spp and seeds are
admitted under an HBM budget and batched into shared wavefronts.  Each
result must be bit-identical whether the request ran alone or in the mix:
every path depends only on (scene, resolution, pixel, sample index, seed).
The plain render path (psy_render_image at the scene's own resolution)
gives the same image as a served request, tying serving to the renderer
the parity tests check against the oracle."""
import numpy as np
import pytest

from psychopath_gb300 import abi, gpu

from . import scene_cases as sc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes3(gpu_lib):
    s = [gpu.Scene(sc.cornell(32, 32, 4, 4)), gpu.Scene(sc.sphere_small(24, 16, 4, 6, level=3)),
         gpu.Scene(sc.motion_small(24, 16, 4, 2))]
    yield s
    for x in s:
        x.close()


def _mix(seed=3, n=24):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        lane = int(rng.integers(0, 3))
        w, h = [(16, 16), (32, 24), (40, 40), (24, 16)][int(rng.integers(0, 4))]
        spp = [1, 2, 4, 8][int(rng.integers(0, 4))]
        out.append((lane, w, h, spp, int(rng.integers(0, 1000))))
    return out


def _server(scenes, **kw):
    srv = gpu.Server(**kw)
    lanes = [srv.add_scene(s) for s in scenes]
    return srv, lanes


def test_request_same_alone_and_in_mix(scenes3):
    reqs = _mix()
    # small waves so that rows of several requests share each wave and a
    # request spans several waves
    srv, lanes = _server(scenes3, wave_paths=4096, waves_in_flight=2)
    alone = []
    for (lane, w, h, spp, seed) in reqs:
        rid = srv.submit(lanes[lane], w, h, spp, seed)
        st = srv.wait(rid)
        assert st["state"] == abi.PSY_REQ_DONE, st
        alone.append(srv.result(rid).copy())
    ids = [srv.submit(lanes[l], w, h, spp, seed) for (l, w, h, spp, seed) in reqs]
    shared = 0
    for i, rid in enumerate(ids):
        st = srv.wait(rid)
        assert st["state"] == abi.PSY_REQ_DONE, st
        assert st["samples"] == reqs[i][1] * reqs[i][2] * reqs[i][3]
        shared += st["shared_waves"]
        got = srv.result(rid)
        assert np.isfinite(got).all()
        assert np.array_equal(got, alone[i]), "request %d differs alone vs in the mix" % i
    assert shared > 0, "no wave carried more than one request"
    stats = srv.stats()
    assert stats["requests_done"] == 2 * len(reqs)
    assert stats["hbm_peak_bytes"] <= stats["hbm_budget_bytes"]
    srv.close()


def test_shortest_policy_same_images_small_first(scenes3):
    """PSY_SCHED_SHORTEST: every image is bit-identical to the FIFO server's;
    small requests submitted right after a large one finish before it (the
    large one has rows left after the first wave), and with a short aging
    bound the large request is not starved (it still finishes while small
    requests keep arriving)."""
    s = scenes3[1]
    big = (s.width * 4, s.height * 4, 16, 5)
    smalls = [(16, 8, 1, 10 + k) for k in range(6)]
    srv, lanes = _server([s], wave_paths=4096)
    ref = {}
    for r in [big] + smalls:
        rid = srv.submit(lanes[0], *r)
        assert srv.wait(rid)["state"] == abi.PSY_REQ_DONE
        ref[r] = srv.result(rid).copy()
    srv.close()
    for aging in (60000, 1):
        srv, lanes = _server([s], wave_paths=4096, policy="shortest", aging_ms=aging, waves_in_flight=1)
        ids = [srv.submit(lanes[0], *r) for r in [big] + smalls]
        sts = [srv.wait(rid) for rid in ids]
        assert all(st["state"] == abi.PSY_REQ_DONE for st in sts)
        for rid, r in zip(ids, [big] + smalls):
            assert np.array_equal(srv.result(rid), ref[r])
        if aging == 60000:  # no aging within the test: strictly shortest first
            assert max(st["latency_s"] for st in sts[1:]) < sts[0]["latency_s"]
        srv.close()


def test_served_request_equals_plain_render(scenes3):
    """A request at the scene's own resolution, spp and seed gives exactly
    the image of psy_render_image; graphs on or off."""
    s = scenes3[1]
    ref, _ = gpu.Renderer(s).render()
    for graphs in (False, True):
        srv, lanes = _server([s], wave_paths=8192, use_graphs=graphs)
        rid = srv.submit(lanes[0], s.width, s.height, s.spp, s.data.seed)
        other = srv.submit(lanes[0], 16, 8, 2, 9)
        assert srv.wait(rid)["state"] == abi.PSY_REQ_DONE
        assert srv.wait(other)["state"] == abi.PSY_REQ_DONE
        assert np.array_equal(srv.result(rid), ref)
        srv.close()


def test_device_output_and_sized_plain_render(scenes3):
    """d_xyz_out requests write the caller's device buffer; the plain render
    path at the same (resolution, spp, seed) gives the same image."""
    torch = pytest.importorskip("torch")
    s = scenes3[0]
    w, h, spp, seed = 40, 24, 4, 77
    ref = torch.zeros(h * w * 3, dtype=torch.float32, device="cuda")
    s.render_sized(w, h, spp, seed, ref.data_ptr())
    d = torch.full((h * w * 3,), -1.0, dtype=torch.float32, device="cuda")
    srv, lanes = _server([s], wave_paths=2048)
    rid = srv.submit(lanes[0], w, h, spp, seed, d_out=d.data_ptr())
    assert srv.wait(rid)["state"] == abi.PSY_REQ_DONE
    torch.cuda.synchronize()
    assert torch.equal(d, ref)
    srv.close()


def test_budget_admission_serialises_images(scenes3):
    """A budget with room for one request image at a time: every request
    still finishes, later ones wait in the queue, and the peak stays within
    the budget."""
    s = scenes3[0]
    probe = gpu.Server(wave_paths=4096)
    probe.add_scene(s)
    base = probe.stats()["hbm_used_bytes"]
    probe.close()
    img = 32 * 32 * 12
    srv, lanes = _server([s], wave_paths=4096, hbm_budget_bytes=base + img + img // 2)
    ids = [srv.submit(lanes[0], 32, 32, 2, k) for k in range(6)]
    sts = [srv.wait(r) for r in ids]
    assert all(st["state"] == abi.PSY_REQ_DONE for st in sts)
    assert max(st["queued_s"] for st in sts[1:]) > 0.0
    stats = srv.stats()
    assert stats["hbm_peak_bytes"] <= base + img + img // 2
    assert stats["hbm_used_bytes"] == base
    srv.close()


def test_cancel_and_errors(scenes3):
    s = scenes3[2]
    srv, lanes = _server([s], wave_paths=2048, max_active=1)
    big = srv.submit(lanes[0], 64, 64, 8, 1)
    queued = srv.submit(lanes[0], 16, 16, 1, 2)
    srv.cancel(queued)
    srv.cancel(big)
    assert srv.wait(queued)["state"] == abi.PSY_REQ_CANCELLED
    assert srv.wait(big)["state"] in (abi.PSY_REQ_CANCELLED, abi.PSY_REQ_DONE)
    # the server keeps serving after cancellations
    ok = srv.submit(lanes[0], 16, 16, 1, 3)
    assert srv.wait(ok)["state"] == abi.PSY_REQ_DONE
    with pytest.raises(gpu.PsyError) as e:
        srv.cancel(ok)
    assert e.value.code == abi.PSY_E_INVALID
    with pytest.raises(gpu.PsyError) as e:
        srv.submit(7, 16, 16, 1, 0)  # unknown lane
    assert e.value.code == abi.PSY_E_INVALID
    with pytest.raises(gpu.PsyError) as e:
        srv.submit(lanes[0], 1024, 4, 4, 0)  # one row exceeds the 2048-path wave
    assert e.value.code == abi.PSY_E_INVALID
    with pytest.raises(gpu.PsyError) as e:
        srv.poll(123456)
    assert e.value.code == abi.PSY_E_NOTFOUND
    srv.close()
