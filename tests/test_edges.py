"""Edge cases of the traversal path: empty and tiny meshes, leaves at the
16-triangle maximum, degenerate triangles, ray batches of 0, 1 and sizes
around the warp width and the 65,536-ray reordering threshold, rays with
zero direction components and tmax 0 or negative, and the 2^23-triangle
limit of the reference's leaf encoding (qbvh.LeafBase).

CPU tests check the builds against the oracle's node arrays and the C-ABI's
validation (no device work); GPU tests compare every hit with the oracle bit
for bit.
"""
import ctypes

import numpy as np
import pytest

import vermeer_gb300 as vg
from vermeer_gb300 import _lib, scenes

from conftest import assert_hits_equal

INVALID = -1


def _export_same(ctx, g, om):
    got = ctx.mesh_export(g)
    ref = om.export()
    for k in ("nodes", "accel_idx"):
        if k in ref:
            assert np.asarray(got[k]).tobytes() == np.asarray(ref[k]).tobytes(), k


def _degenerate_mesh():
    """Collinear, repeated-vertex and zero-area triangles among ordinary ones."""
    v, ip = scenes.triangle_soup(300, 61, edge=0.05)
    v = v.copy()
    v[3 * 5 + 1] = v[3 * 5]                    # two equal vertices
    v[3 * 6 + 2] = 0.5 * (v[3 * 6] + v[3 * 6 + 1])  # collinear
    v[3 * 7 + 1] = v[3 * 7 + 2] = v[3 * 7]     # a point
    return v.astype(np.float32), ip


@pytest.mark.parametrize("n_tris", [1, 2, 15, 16, 17, 33])
def test_tiny_meshes_build_like_the_oracle(host_ctx, orc, n_tris):
    """One leaf holds up to 16 triangles (leafMax 16): 16 stays one leaf, 17
    splits; every build equals the oracle's BuildAccel."""
    v, ip = scenes.triangle_soup(n_tris, 60 + n_tris, edge=0.05)
    g = host_ctx.mesh_build(v, ip)
    _export_same(host_ctx, g, orc.Mesh(v, ip))


def test_degenerate_triangles_build_like_the_oracle(host_ctx, orc):
    v, ip = _degenerate_mesh()
    g = host_ctx.mesh_build(v, ip)
    _export_same(host_ctx, g, orc.Mesh(v, ip))


def test_mesh_input_validation(host_ctx):
    L = host_ctx.L
    verts = np.zeros((3, 3), np.float32)
    idxp = np.array([0, 1, 5], np.uint32)  # index out of range
    g = ctypes.c_uint32()
    mi = _lib.MeshInput(verts.ctypes.data_as(ctypes.c_void_p), 3, 1, idxp.ctypes.data_as(ctypes.c_void_p), 1,
                        0.0, 0, None)
    assert L.vmr_mesh_build(host_ctx.h, ctypes.byref(mi), ctypes.byref(g)) == INVALID
    assert b"out of range" in L.vmr_last_error(host_ctx.h)
    # the leaf encoding's 23-bit base (checked before the indices are read)
    mi = _lib.MeshInput(verts.ctypes.data_as(ctypes.c_void_p), 3, 1, idxp.ctypes.data_as(ctypes.c_void_p), 1 << 23,
                        0.0, 0, None)
    assert L.vmr_mesh_build(host_ctx.h, ctypes.byref(mi), ctypes.byref(g)) == INVALID
    assert b"2^23" in L.vmr_last_error(host_ctx.h)
    mi = _lib.MeshInput(None, 0, 0, None, 0, 0.0, 0, None)  # zero motion keys
    assert L.vmr_mesh_build(host_ctx.h, ctypes.byref(mi), ctypes.byref(g)) == INVALID


# ------------------------------------------------------------------ GPU ----
def _awkward_rays(n, seed):
    """Incoherent rays with every kind of awkward component mixed in."""
    r = scenes.incoherent_rays(n, seed)
    k = max(1, n // 8)
    r[:k, 3] = 0.0                      # D.x = 0
    r[k:2 * k, 4:6] = 0.0               # D along x only
    r[k:2 * k, 3] = np.where(np.arange(k) % 2 == 0, 1.0, -1.0)
    r[2 * k:3 * k, 6] = 0.0             # tmax 0
    r[3 * k:4 * k, 6] = -1.0            # negative tmax
    r[4 * k:5 * k, 6] = 0.05            # short rays
    r[5 * k:6 * k, 3:6] = -r[5 * k:6 * k, 3:6]
    return r


@pytest.mark.gpu
@pytest.mark.parametrize("n_rays", [0, 1, 31, 32, 33, 65535, 65536, 65537])
def test_ray_batch_sizes(ctx, orc, n_rays):
    """Batches around the warp width and the reordering threshold (65,536
    rays): hits equal the oracle's, closest and any hit, host and device
    pointers; an empty batch is a no-op."""
    import torch
    v, ip = scenes.triangle_soup(20000, 62, edge=0.01)
    g = ctx.mesh_build(v, ip)
    om = orc.Mesh(v, ip)
    rays = _awkward_rays(n_rays, 63) if n_rays else np.zeros((0, 8), np.float32)
    for shadow in (False, True):
        got = ctx.trace_mesh(g, rays, shadow=shadow)
        assert got["stats"]["rays"] == n_rays
        if n_rays == 0:
            assert got["prim"].size == 0
            continue
        ref = om.trace(rays, shadow=shadow)
        if shadow:
            assert np.array_equal(got["prim"] >= 0, ref["prim"] >= 0)
        else:
            assert_hits_equal(got, ref, what=f"n={n_rays}")
        dev = torch.from_numpy(np.ascontiguousarray(rays.T)).cuda()
        d = ctx.trace_mesh(g, dev, shadow=shadow)
        ctx.sync()
        assert np.array_equal(d["prim"].cpu().numpy(), got["prim"])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["one_triangle", "one_full_leaf", "degenerate"])
def test_small_and_degenerate_meshes_trace_like_the_oracle(ctx, orc, kind):
    if kind == "one_triangle":
        v, ip = scenes.triangle_soup(1, 64, edge=0.4)
    elif kind == "one_full_leaf":
        v, ip = scenes.triangle_soup(16, 65, edge=0.3)
    else:
        v, ip = _degenerate_mesh()
    g = ctx.mesh_build(v, ip)
    om = orc.Mesh(v, ip)
    rays = _awkward_rays(70000, 66)
    # aim a share of the rays at vertices and edge midpoints
    tv = v.reshape(-1, 3, 3)
    pick = tv[np.arange(20000) % tv.shape[0]]
    tgt = np.where((np.arange(20000) % 2 == 0)[:, None], pick[:, 0], 0.5 * (pick[:, 1] + pick[:, 2]))
    d = tgt - rays[:20000, :3]
    rays[:20000, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:20000, 6] = np.inf
    for shadow in (False, True):
        got = ctx.trace_mesh(g, rays, shadow=shadow)
        ref = om.trace(rays, shadow=shadow)
        if shadow:
            assert np.array_equal(got["prim"] >= 0, ref["prim"] >= 0)
        else:
            assert_hits_equal(got, ref, what=kind)
