"""One image over several GPUs (vmr_render_split, vmr_render_path_split and
the process-group form vermeer_gb300.shard): the rows are cut into one band
per device, each band samples its pixels exactly as the whole render does,
and the bands are put together; the image must be the one-device image bit
for bit (each pixel's running mean is folded by one device only, as each
pixel of the reference's tiles is folded by one worker, core/render.go:66-131).

CPU tests run the partition and the gather with world size 2 on gloo, each
rank rendering its band with the oracle; GPU tests split a render over two
contexts on the one GPU (the same code path as two GPUs: one host thread and
stream per context) and compare with the one-context render.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import vermeer_gb300 as vg  # noqa: E402
from vermeer_gb300 import scenes  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_split_rows_partition():
    for h in (1, 2, 7, 255, 1080):
        for n in (1, 2, 3, 4, 8, 9):
            b = vg.split_rows(h, n)
            assert len(b) == n
            assert b[0][0] == 0 and sum(c for _, c in b) == h
            for (r0, c0), (r1, _) in zip(b, b[1:]):
                assert r1 == r0 + c0  # contiguous, in order
            counts = [c for _, c in b]
            assert max(counts) - min(counts) <= 1


W, H = 40, 23  # an odd height: the bands differ by one row


def _rank(rank, world, port, out, kind):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import orc
    from vermeer_gb300 import scenes, shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r0, n = shard.band(H, rank, world)
        if kind == "reference":
            r = orc.Render(scenes.small_room(1024, seed=3))
            fb = r.run(W, H, 0, 3, 9, rows=(r0, n), nthreads=2)
        else:
            r = orc.Render(scenes.small_room_ext(1024, seed=3))
            fb, fb64 = r.run_path(W, H, 0, 3, 9, max_depth=5, rows=(r0, n), nthreads=2)
            fb = np.concatenate([fb, fb64.astype(np.float32)], axis=-1)  # both buffers through the gather
        img = shard.gather_image(fb, H, W)
        out[rank] = img.tobytes()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind", ["reference", "path"])
def test_two_gloo_ranks_gather_the_one_device_image(orc, kind):
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, out, kind), nprocs=world, start_method="spawn", join=True)
        got = dict(out)
    assert got[0] == got[1]
    if kind == "reference":
        ref = orc.Render(scenes.small_room(1024, seed=3)).run(W, H, 0, 3, 9)
    else:
        fb, fb64 = orc.Render(scenes.small_room_ext(1024, seed=3)).run_path(W, H, 0, 3, 9, max_depth=5)
        ref = np.concatenate([fb, fb64.astype(np.float32)], axis=-1)
    img = np.frombuffer(got[0], np.float32).reshape(ref.shape)
    assert img.tobytes() == ref.tobytes()


def test_oracle_bands_equal_the_whole(orc):
    """The band renders themselves (no gather): every band of a 3-way split
    is the matching rows of the whole image."""
    r = orc.Render(scenes.small_room(1024, seed=4))
    whole = r.run(W, H, 0, 2, 5)
    for r0, n in vg.split_rows(H, 3):
        assert r.run(W, H, 0, 2, 5, rows=(r0, n)).tobytes() == whole[r0:r0 + n].tobytes()


@pytest.mark.gpu
def test_split_over_two_contexts_is_the_one_context_image(ctx):
    sc = scenes.small_room(4096, seed=5)
    ctx.load_scene(sc)
    one, _ = ctx.render(64, 47, 0, 4, 3)
    other = vg.Context(0)
    try:
        other.load_scene(sc)
        got, st = vg.render_split([ctx, other], 64, 47, 0, 4, 3)
        assert got.tobytes() == one.tobytes()
        assert st["samples"] == 64 * 47 * 4
        # a band alone is the matching rows
        band, _ = other.render(64, 47, 0, 4, 3, rows=(10, 20))
        assert band.tobytes() == one[10:30].tobytes()
    finally:
        other.close()


@pytest.mark.gpu
def test_path_split_over_two_contexts_is_the_one_context_image(ctx):
    sc = scenes.small_room_ext(4096, seed=6)
    ctx.load_scene(sc)
    one, _ = ctx.render_path(64, 47, 0, 4, 3, max_depth=5)
    other = vg.Context(0)
    try:
        other.load_scene(sc)
        got, st = vg.render_path_split([ctx, other], 64, 47, 0, 4, 3, max_depth=5)
        assert got.tobytes() == one.tobytes()
        band, _ = other.render_path(64, 47, 0, 4, 3, max_depth=5, rows=(5, 17))
        assert band.tobytes() == one[5:22].tobytes()
    finally:
        other.close()
