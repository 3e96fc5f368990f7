"""vmr_trace_mesh_noalloc: the mesh trace for callers that must not have a
library allocate device memory while they run (a host that sub-allocates the
whole device itself, or a frame loop with no room for cudaMalloc's
synchronisation).  Its scratch is one static device array, so the tests check
that two calls in a row each give exactly the hits of the allocating entry
point (vmr_trace_mesh on device buffers) and of the oracle, again after the
mesh was autotuned (its own kernel, block size and sort-key width), that a
warmed-up call leaves the device's free memory unchanged, that batches below
the reordering threshold work too, and that oversized batches and host
pointers are refused before any launch."""
import ctypes

import numpy as np
import pytest

from conftest import assert_hits_equal

FIELDS = ("prim", "t", "u", "v", "w")
TRACE_ANY_HIT, TRACE_DEVICE = 1, 2


def _device_rays(rays):
    import torch
    return torch.from_numpy(np.ascontiguousarray(rays.T)).cuda()


def _outputs(n, device):
    import torch
    return {k: torch.full((n,), 7, dtype=torch.int32 if k == "prim" else torch.float32, device=device)
            for k in FIELDS}


def _call(ctx, geom, d_rays, out, flags):
    from vermeer_gb300 import _lib
    P = ctypes.c_void_p
    n = d_rays.shape[1]
    r = _lib.Rays(*[P(d_rays[k].data_ptr()) for k in range(8)])
    h = _lib.Hits(P(out["prim"].data_ptr()), None, *[P(out[k].data_ptr()) for k in ("t", "u", "v", "w")])
    rc = ctx.L.vmr_trace_mesh_noalloc(ctx.h, geom, ctypes.byref(r), n, flags, ctypes.byref(h))
    return rc, ctx.L.vmr_last_error(ctx.h).decode()


def _noalloc(ctx, geom, d_rays, shadow):
    out = _outputs(d_rays.shape[1], d_rays.device)
    rc, msg = _call(ctx, geom, d_rays, out, (TRACE_ANY_HIT if shadow else 0) | TRACE_DEVICE)
    return rc, msg, {k: out[k].cpu().numpy() for k in FIELDS}


def _reference(ctx, geom, d_rays, shadow):
    ref = ctx.trace_mesh(geom, d_rays, shadow=shadow)
    ctx.sync()
    return {k: ref[k].cpu().numpy() for k in FIELDS}


@pytest.mark.gpu
@pytest.mark.parametrize("n_rays", [200000, 5000])
def test_noalloc_equals_trace_mesh_and_oracle_on_two_calls(ctx, orc, n_rays):
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(200000, 23, edge=0.006)
    geom = ctx.mesh_build(v, ip)
    om = orc.Mesh(v, ip)
    rays = scenes.incoherent_rays(n_rays, 24)
    d_rays = _device_rays(rays)
    for shadow in (False, True):
        ref = _reference(ctx, geom, d_rays, shadow)
        if not shadow:  # closest hit is unique; any-hit prims depend on the tuning's order
            assert_hits_equal(ref, om.trace(rays, shadow=False), what=f"trace_mesh vs oracle n={n_rays}")
        for call in range(2):
            rc, msg, got = _noalloc(ctx, geom, d_rays, shadow)
            assert rc == 0, msg
            assert_hits_equal(got, ref, what=f"noalloc call {call} shadow={shadow} n={n_rays}")


@pytest.mark.gpu
def test_noalloc_follows_the_autotuned_mesh_and_allocates_nothing(ctx, orc):
    """After vmr_autotune the mesh traces with its own tuning; the no-alloc
    call must use it too (same kernel, block size and sort-key width), and a
    warmed-up call must not change the device's free memory."""
    import torch
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(150000, 27, edge=0.006)
    geom = ctx.mesh_build(v, ip)
    om = orc.Mesh(v, ip)
    rays = scenes.incoherent_rays(250000, 28)
    d_rays = _device_rays(rays)
    try:
        ctx.autotune(geom, d_rays[:, :200000].contiguous())
        expect = om.trace(rays, shadow=False)
        ref_any = _reference(ctx, geom, d_rays, True)
        outs = [_outputs(d_rays.shape[1], d_rays.device) for _ in range(3)]
        rc, msg = _call(ctx, geom, d_rays, outs[0], TRACE_DEVICE)  # warm-up
        assert rc == 0, msg
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc, msg = _call(ctx, geom, d_rays, outs[1], TRACE_DEVICE)
        assert rc == 0, msg
        rc, msg = _call(ctx, geom, d_rays, outs[2], TRACE_DEVICE | TRACE_ANY_HIT)
        assert rc == 0, msg
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0
        for k in range(2):
            got = {f: outs[k][f].cpu().numpy() for f in FIELDS}
            assert_hits_equal(got, expect, what=f"autotuned noalloc call {k} vs oracle")
        got = {f: outs[2][f].cpu().numpy() for f in FIELDS}
        assert_hits_equal(got, ref_any, what="autotuned noalloc any-hit vs trace_mesh")
    finally:
        ctx.clear_tuning(geom)


@pytest.mark.gpu
def test_noalloc_refuses_oversized_batch(ctx):
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(1000, 25)
    geom = ctx.mesh_build(v, ip)
    rays = scenes.incoherent_rays(262144 + 1, 26)
    rc, msg, _ = _noalloc(ctx, geom, _device_rays(rays), False)
    assert rc == -1 and "VMR_NOALLOC_MAX_RAYS" in msg


@pytest.mark.gpu
def test_noalloc_refuses_host_arrays_on_a_gpu_context(ctx):
    """Host arrays under VMR_TRACE_DEVICE are found by their pointer
    attributes and refused; the output arrays stay untouched."""
    from vermeer_gb300 import _lib, scenes
    v, ip = scenes.triangle_soup(1000, 29)
    geom = ctx.mesh_build(v, ip)
    soa = np.ascontiguousarray(scenes.incoherent_rays(1000, 30).T)
    out = {k: np.full(1000, 7, np.int32 if k == "prim" else np.float32) for k in FIELDS}
    P = ctypes.c_void_p
    r = _lib.Rays(*[P(soa[k].ctypes.data) for k in range(8)])
    h = _lib.Hits(P(out["prim"].ctypes.data), None, *[P(out[k].ctypes.data) for k in ("t", "u", "v", "w")])
    rc = ctx.L.vmr_trace_mesh_noalloc(ctx.h, geom, ctypes.byref(r), 1000, TRACE_DEVICE, ctypes.byref(h))
    assert rc == -1 and "not device memory" in ctx.L.vmr_last_error(ctx.h).decode()
    assert (out["prim"] == 7).all()


def test_noalloc_requires_the_device_flag(host_ctx):
    """Without VMR_TRACE_DEVICE the call is refused before it looks at the
    context or the GPU (here a host-only context, no GPU needed)."""
    from vermeer_gb300 import _lib
    soa = np.zeros((8, 4), np.float32)
    out = {k: np.zeros(4, np.int32 if k == "prim" else np.float32) for k in FIELDS}
    P = ctypes.c_void_p
    r = _lib.Rays(*[P(soa[k].ctypes.data) for k in range(8)])
    h = _lib.Hits(P(out["prim"].ctypes.data), None, *[P(out[k].ctypes.data) for k in ("t", "u", "v", "w")])
    for flags in (0, TRACE_ANY_HIT):
        rc = host_ctx.L.vmr_trace_mesh_noalloc(host_ctx.h, 0, ctypes.byref(r), 4, flags, ctypes.byref(h))
        assert rc == -1
        assert "VMR_TRACE_DEVICE" in host_ctx.L.vmr_last_error(host_ctx.h).decode()
