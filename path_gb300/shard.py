"""One image over several GPUs: row bands per rank, gathered on rank 0.

A render has no data-path exchange: every pixel is computed on its own.
Each rank renders a contiguous band of rows (``SquareImage(rows=...)``), cut
at the render WorkDivision's y-block boundaries so no CTA is split between
ranks, and rank 0 assembles the bands with one ``torch.distributed.gather``
of host tensors (gloo or NCCL process group; with NCCL the bands travel as
CUDA tensors).  Band pixels are bit-identical to the single-GPU render, so
the gathered image is too.  On one GPU this is a no-op (world size 1).
"""

import numpy as np

from . import api


def band_rows(rank, world, y_dim, y_block_size):
    """Rows [start, end) of ``rank``'s band: y blocks dealt out evenly,
    the first ranks taking one more when they do not divide."""
    n_yb = (y_dim + y_block_size - 1) // y_block_size
    per, extra = divmod(n_yb, world)
    b0 = rank * per + min(rank, extra)
    b1 = b0 + per + (1 if rank < extra else 0)
    return min(b0 * y_block_size, y_dim), min(b1 * y_block_size, y_dim)


def render_band(renderer, scene, settings, spp, x_dim, y_dim, film_to_world, rank, world):
    """This rank's band of a FloatRGB render: (image [y_dim, x_dim, 3] with
    only the band filled, (row_start, row_end))."""
    wd = api.work_division(settings.render_work_division, spp, x_dim, y_dim)
    lo, hi = band_rows(rank, world, y_dim, wd["y_block_size"])
    img = np.zeros((y_dim, x_dim, 3), np.float32)
    if hi > lo:
        renderer.render(api.ExecutionModel.GPU, api.SquareImage(x_dim, y_dim, film_to_world,
                                                                rows=(lo, hi)),
                        img, scene, spp, settings)
    return img, (lo, hi)


def gather_bands(img, rows, rank, world, dst=0, device=None):
    """Assemble every rank's band on ``dst``; returns the full image there
    and None elsewhere.  ``img`` is this rank's [H, W, 3] float32 image."""
    import torch
    import torch.distributed as dist
    if world == 1:
        return img
    t = torch.from_numpy(np.ascontiguousarray(img))
    if device is not None:
        t = t.to(device)
    bounds = torch.tensor([rows[0], rows[1]], dtype=torch.int64, device=t.device)
    all_bounds = [torch.zeros_like(bounds) for _ in range(world)] if rank == dst else None
    dist.gather(bounds, all_bounds, dst=dst)
    all_imgs = [torch.zeros_like(t) for _ in range(world)] if rank == dst else None
    dist.gather(t, all_imgs, dst=dst)
    if rank != dst:
        return None
    out = np.zeros_like(img)
    for b, im in zip(all_bounds, all_imgs):
        lo, hi = int(b[0]), int(b[1])
        out[lo:hi] = im.cpu().numpy()[lo:hi]
    return out
