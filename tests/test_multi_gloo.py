"""Host logic of the multi-GPU row split (psychopath_gb300/multi.py): the
bands cover every row once, and the all-gather reassembles the full image
from the ranks' bands -- run as 2 and 3 gloo ranks on CPU."""
import os
import socket

import numpy as np
import pytest

from psychopath_gb300 import multi


def test_row_bands_cover_rows_once():
    for h in (1, 7, 1080):
        for world in (1, 2, 3, 8):
            bands = multi.row_bands(h, world)
            assert len(bands) == world
            assert bands[0][0] == 0 and bands[-1][1] == h
            assert all(a[1] == b[0] for a, b in zip(bands, bands[1:]))
            sizes = [b1 - b0 for b0, b1 in bands]
            assert max(sizes) - min(sizes) <= 1
    assert multi.band_crop((10, 20), 64) == (0, 10, 63, 19)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, h, w, out_dir):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    full = torch.arange(h * w * 3, dtype=torch.float32).reshape(h, w, 3)
    bands = multi.row_bands(h, world)
    img = torch.full((h, w, 3), -1.0)  # rows outside this rank's band are garbage
    y0, y1 = bands[rank]
    img[y0:y1] = full[y0:y1]
    got = multi.gather_bands(img, bands, rank, world)
    np.save(os.path.join(out_dir, "r%d.npy" % rank), got.numpy())
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gather_bands_gloo(tmp_path, world):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    h, w = 11, 5
    mp.start_processes(_worker, args=(world, _free_port(), h, w, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    full = np.arange(h * w * 3, dtype=np.float32).reshape(h, w, 3)
    for r in range(world):
        assert np.array_equal(np.load(tmp_path / ("r%d.npy" % r)), full)
