"""Host logic of the multi-GPU frame split (psychopath_gb300/multi.py), run as
2 and 3 gloo ranks on CPU: each rank renders its interleaved rows of a frame
(here with the CPU oracle standing in for its GPU), the all-gather puts the
rows together, and the gathered image equals a one-rank render of the whole
frame (every pixel depends only on its own paths).  The oracle adds a
bucket's samples into a pixel in its path-compaction order, as the reference
does, and that order depends on the bucket's other paths, so a pixel can
differ by the last ulps of that sum (1e-6 relative here); every path itself
is identical."""
import os
import socket

import numpy as np
import pytest

from psychopath_gb300 import multi


def test_interleaved_rows_cover_rows_once():
    for h in (1, 7, 1080):
        for world in (1, 2, 3, 8):
            seen = sorted(y for r in range(world) for y in multi.rows_of(h, world, r))
            assert seen == list(range(h))
            counts = [len(multi.rows_of(h, world, r)) for r in range(world)]
            assert max(counts) - min(counts) <= 1 and max(counts) == multi.max_rows(h, world)
    with pytest.raises(ValueError):
        multi.rows_of(10, 2, 2)


def test_row_bands_cover_rows_once():
    for h in (1, 7, 1080):
        for world in (1, 2, 3, 8):
            bands = multi.row_bands(h, world)
            assert bands[0][0] == 0 and bands[-1][1] == h
            assert all(a[1] == b[0] for a, b in zip(bands, bands[1:]))
    assert multi.band_crop((10, 20), 64) == (0, 10, 63, 19)


def test_interleaving_balances_a_centred_load():
    """Per-row cost concentrated in the middle of the frame (an object in the
    centre, as the mesh-stress frame): interleaved rows give every rank
    nearly the same share, contiguous bands do not."""
    h, world = 1080, 8
    cost = np.exp(-((np.arange(h) - h / 2) / (h / 8)) ** 2) + 0.05
    inter = [cost[list(multi.rows_of(h, world, r))].sum() for r in range(world)]
    bands = [cost[b0:b1].sum() for b0, b1 in multi.row_bands(h, world)]
    assert max(inter) / min(inter) < 1.02
    assert max(bands) / min(bands) > 5


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _scene():
    from tests import scene_cases as sc
    return sc.cornell(16, 11, 4, 2)


def _worker(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    import torch.distributed as dist
    from oracle.runner import OracleScene
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sd = _scene()
    o = OracleScene(sd)
    W, H = sd.width, sd.height
    rows = list(multi.rows_of(H, world, rank))
    mine = np.zeros((len(rows), W, 3), dtype=np.float32)
    for k, y in enumerate(rows):  # this rank's rows, each one a crop of the frame
        img, _ = o.render(threads=1, crop=(0, y, W - 1, y))
        mine[k] = img[y]
    got = multi.gather_rows(torch.from_numpy(mine), H, rank, world)
    np.save(os.path.join(out_dir, "r%d.npy" % rank), got.numpy())
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_interleaved_render_gathers_to_the_whole_frame(tmp_path, world):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle.runner import OracleScene
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    full, _ = OracleScene(_scene()).render(threads=1)
    for r in range(world):
        got = np.load(tmp_path / ("r%d.npy" % r))
        assert np.allclose(got, full, rtol=1e-6, atol=0.0)
    assert full.min() >= 0.0 and (full > 0).mean() > 0.9
