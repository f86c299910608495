"""Multi-GPU partitioning of one render: one process per GPU, each renders a
band of whole pixel rows of the same frame (same seed, so every pixel is
the one a single-GPU render produces: paths are independent per pixel and
sample), and one all-gather at the end puts the bands together.  No
collective inside the render.

The reference parallelises the same way over buckets on CPU threads
(Renderer::render, src/renderer.rs:76-191): independent pixel regions,
one shared image.
"""


def row_bands(height, world):
    """[y0, y1) row ranges for `world` ranks, covering 0..height once, sizes
    differing by at most one row."""
    if world < 1:
        raise ValueError("world must be >= 1")
    base, extra = divmod(height, world)
    out, y = [], 0
    for r in range(world):
        h = base + (1 if r < extra else 0)
        out.append((y, y + h))
        y += h
    return out


def gather_bands(image, bands, rank, world, group=None):
    """All-gather the ranks' bands of `image` (a torch tensor of shape
    (height, width, 3), each rank holding valid rows only in its own band)
    and return the full image on every rank.  Bands are padded to the
    largest band so every rank sends the same number of elements."""
    import torch
    import torch.distributed as dist
    h, w = image.shape[0], image.shape[1]
    rows = max(b1 - b0 for b0, b1 in bands)
    y0, y1 = bands[rank]
    send = torch.zeros((rows, w, 3), dtype=image.dtype, device=image.device)
    send[: y1 - y0] = image[y0:y1]
    recv = [torch.empty_like(send) for _ in range(world)]
    dist.all_gather(recv, send, group=group)
    out = torch.empty_like(image)
    for r, (b0, b1) in enumerate(bands):
        out[b0:b1] = recv[r][: b1 - b0]
    return out


def band_crop(band, width):
    """The inclusive crop rectangle (x0, y0, x1, y1) psy_render_image_device
    takes for a row band."""
    y0, y1 = band
    return (0, y0, width - 1, y1 - 1)
