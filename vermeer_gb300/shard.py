"""One image rendered by the ranks of a process group (one process per GPU,
launched with torchrun): the reference's tile split of a render
(core/render.go:184-204) across processes.

Each rank renders one contiguous band of rows (the bands of libvmr's
vmr_split_rows), sampling every pixel of the band exactly as the whole render
does, so the running mean of a pixel is folded by one rank only; the bands
are then gathered into the full image on every rank.  The gathered image is
the one-rank render bit for bit: no framebuffer reduction, no change to the
fold.  The single-process form over several contexts is
vermeer_gb300.render_split (vmr_render_split).
"""
from __future__ import annotations

import numpy as np

from .api import split_rows


def band(height: int, rank: int, world: int) -> tuple[int, int]:
    """(row_begin, row_count) of a rank's band."""
    return split_rows(height, world)[rank]


def gather_image(band_fb, height: int, width: int, group=None):
    """The full [height, width, C] image from every rank's band (all_gather
    over the group; bands padded to the tallest).  Works with gloo (CPU
    tensors) and NCCL (the tensors go to the rank's current CUDA device)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    bands = split_rows(height, world)
    tallest = max(c for _, c in bands)
    band_fb = np.ascontiguousarray(band_fb)
    chans = band_fb.shape[-1]
    pad = np.zeros((tallest, width, chans), band_fb.dtype)
    pad[: band_fb.shape[0]] = band_fb
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else None
    t = torch.from_numpy(pad)
    if dev is not None:
        t = t.to(dev)
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    out = np.empty((height, width, chans), band_fb.dtype)
    for (r0, n), part in zip(bands, parts):
        out[r0:r0 + n] = part[:n].cpu().numpy()
    return out


def render_distributed(ctx, width: int, height: int, iter_begin: int, iter_count: int, seed: int,
                       path: bool = False, group=None, **kw):
    """This rank's band rendered by ctx (reference mode, or the extended path
    tracer with path=True and Context.render_path's keyword arguments), then
    the whole image gathered on every rank.  Returns (image, this rank's
    stats)."""
    import torch.distributed as dist
    r0, n = band(height, dist.get_rank(group), dist.get_world_size(group))
    if path:
        fb, st = ctx.render_path(width, height, iter_begin, iter_count, seed, rows=(r0, n), **kw)
    else:
        fb, st = ctx.render(width, height, iter_begin, iter_count, seed, rows=(r0, n), **kw)
    return gather_image(fb, height, width, group), st
