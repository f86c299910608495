"""Multi-GPU partitioning of one render: one process per GPU.  Rank r of N
renders the interleaved image rows r, r + N, r + 2N, ... of the same frame
(psy_render_rows_device; same seed, so every pixel is the one a single-GPU
render produces: paths are independent per pixel and sample), and one
all-gather at the end puts the rows together.  No collective inside the
render.

Interleaving balances the ranks: a frame's expensive pixels (a mesh in the
middle of the image) are spread over every rank, as the reference balances
its CPU threads by handing Hilbert-ordered buckets to whichever thread is
free (Renderer::render, src/renderer.rs:150-180).  Contiguous bands
(row_bands) would give the middle ranks most of the paths.
"""


def rows_of(height, world, rank):
    """The image rows rank `rank` of `world` renders: rank, rank + world, ..."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return range(rank, height, world)


def max_rows(height, world):
    """The most rows any rank holds (rank 0's count)."""
    return len(rows_of(height, world, 0))


def gather_rows(rows_img, height, rank, world, group=None):
    """All-gather the ranks' interleaved rows and return the full image on
    every rank.  rows_img: this rank's rows in order, a torch tensor of shape
    (len(rows_of(height, world, rank)), width, 3) or larger (extra rows are
    ignored).  Every rank sends max_rows(height, world) rows, padded."""
    import torch
    import torch.distributed as dist
    w = rows_img.shape[1]
    n_max = max_rows(height, world)
    n = len(rows_of(height, world, rank))
    send = torch.zeros((n_max, w, 3), dtype=rows_img.dtype, device=rows_img.device)
    send[:n] = rows_img[:n]
    recv = [torch.empty_like(send) for _ in range(world)]
    dist.all_gather(recv, send, group=group)
    out = torch.empty((height, w, 3), dtype=rows_img.dtype, device=rows_img.device)
    for r in range(world):
        out[r::world] = recv[r][: len(rows_of(height, world, r))]
    return out


def row_bands(height, world):
    """[y0, y1) contiguous row ranges for `world` ranks, covering 0..height
    once, sizes differing by at most one row (a crop per rank; unbalanced
    when the image's cost is concentrated, kept for comparison)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    base, extra = divmod(height, world)
    out, y = [], 0
    for r in range(world):
        h = base + (1 if r < extra else 0)
        out.append((y, y + h))
        y += h
    return out


def band_crop(band, width):
    """The inclusive crop rectangle (x0, y0, x1, y1) psy_render_image_device
    takes for a row band."""
    y0, y1 = band
    return (0, y0, width - 1, y1 - 1)
