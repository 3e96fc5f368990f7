"""vmr_trace_mesh_noalloc: the mesh trace for callers that must not have a
library allocate device memory while they run (a host that sub-allocates the
whole device itself, or a frame loop with no room for cudaMalloc's
synchronisation).  Its scratch is one static device array, so the test checks
that two calls in a row each give exactly the hits of the allocating entry
point (vmr_trace_mesh on device buffers), that batches below the reordering
threshold work too, and that an oversized batch is refused."""
import ctypes

import numpy as np
import pytest

from conftest import assert_hits_equal

pytestmark = pytest.mark.gpu

FIELDS = ("prim", "t", "u", "v", "w")


def _device_rays(rays):
    import torch
    return torch.from_numpy(np.ascontiguousarray(rays.T)).cuda()


def _noalloc(ctx, geom, d_rays, shadow):
    import torch
    from vermeer_gb300 import _lib
    n = d_rays.shape[1]
    out = {k: torch.full((n,), 7, dtype=torch.int32 if k == "prim" else torch.float32, device=d_rays.device)
           for k in FIELDS}
    P = ctypes.c_void_p
    r = _lib.Rays(*[P(d_rays[k].data_ptr()) for k in range(8)])
    h = _lib.Hits(P(out["prim"].data_ptr()), None, *[P(out[k].data_ptr()) for k in ("t", "u", "v", "w")])
    flags = (1 if shadow else 0) | 2
    rc = ctx.L.vmr_trace_mesh_noalloc(ctx.h, geom, ctypes.byref(r), n, flags, ctypes.byref(h))
    msg = ctx.L.vmr_last_error(ctx.h).decode()
    return rc, msg, {k: out[k].cpu().numpy() for k in FIELDS}


@pytest.mark.parametrize("n_rays", [200000, 5000])
def test_noalloc_equals_trace_mesh_on_two_calls(ctx, n_rays):
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(200000, 23, edge=0.006)
    geom = ctx.mesh_build(v, ip)
    rays = scenes.incoherent_rays(n_rays, 24)
    d_rays = _device_rays(rays)
    for shadow in (False, True):
        ref = ctx.trace_mesh(geom, d_rays, shadow=shadow)
        ctx.sync()
        ref = {k: ref[k].cpu().numpy() for k in FIELDS}
        for call in range(2):
            rc, msg, got = _noalloc(ctx, geom, d_rays, shadow)
            assert rc == 0, msg
            assert_hits_equal(got, ref, what=f"noalloc call {call} shadow={shadow} n={n_rays}")


def test_noalloc_refuses_oversized_batch(ctx):
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(1000, 25)
    geom = ctx.mesh_build(v, ip)
    rays = scenes.incoherent_rays(262144 + 1, 26)
    rc, msg, _ = _noalloc(ctx, geom, _device_rays(rays), False)
    assert rc == -1 and "VMR_NOALLOC_MAX_RAYS" in msg
