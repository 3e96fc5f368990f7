"""The device QBVH builder (gpubuild.cu, vmr_set_builder(VMR_BUILD_DEVICE))
gives the oracle's node arrays, leaf order and bounds byte for byte: the
reference builder qbvh.BuildAccel (qbvh/build.go:28-307) as
PolyMesh.initAccel runs it (builtin/geom/polymesh/buildqbvh.go:14-144).

The CPU tests check the closed form of the reference's in-place partition
(build.go:111-130) that the device builder evaluates with prefix counts."""
import numpy as np
import pytest

import vermeer_gb300 as vg
from vermeer_gb300 import scenes

from test_builder_parity import _soups


def _reference_partition(right):
    """build.go:111-130 on a list of 'right' flags; returns the permutation."""
    a = list(range(len(right)))
    lo, hi = 0, len(a) - 1
    while lo <= hi:
        if not right[a[lo]]:
            lo += 1
        else:
            a[lo], a[hi] = a[hi], a[lo]
            hi -= 1
    return a, lo


def _closed_form(right):
    """The permutation the device builder computes (gpubuild.cu)."""
    n = len(right)
    nl = n - sum(right)
    p = nl + (1 if nl < n and right[nl] else 0)
    lsw = [k for k in range(p) if right[k]]
    rsw = [i for i in range(n - 1, p - 1, -1) if not right[i]]
    out = [None] * n
    for k in range(p):
        if not right[k]:
            out[k] = k
    for j, k in enumerate(lsw):
        out[n - 1 if j == 0 else rsw[j - 1] - 1] = k
    for i in range(p, n):
        if right[i]:
            out[i - 1] = i
    for r, i in enumerate(rsw):
        out[lsw[r]] = i
    return out, nl


def test_partition_closed_form_matches_reference_partition():
    rng = np.random.default_rng(5)
    for _ in range(20000):
        n = int(rng.integers(0, 40))
        right = list(rng.random(n) < rng.random())
        assert _closed_form(right) == _reference_partition(right), right


@pytest.fixture()
def dev_ctx(ctx):
    ctx.set_builder(vg.BUILD_DEVICE)
    yield ctx
    ctx.set_builder(vg.BUILD_AUTO)


def _check_static(orc, ctx, v, ip, name):
    ref = orc.Mesh(v, ip).export()
    g = ctx.mesh_build(v, ip)
    got = ctx.mesh_export(g)
    assert got["nodes"].tobytes() == ref["nodes"].tobytes(), name
    assert np.array_equal(got["accel_idx"], ref["accel_idx"]), name
    assert np.array_equal(got["idxp"], ref["idxp"]), name
    assert np.array_equal(got["bounds"].view(np.uint32), ref["bounds"].view(np.uint32)), name
    return g


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(range(8)))
def test_device_build_matches_oracle(orc, dev_ctx, case):
    name, v, ip = list(_soups())[case]
    _check_static(orc, dev_ctx, v, ip, name)


@pytest.mark.gpu
def test_device_build_signed_zeros_and_ties(orc, dev_ctx):
    """Coordinates of +0 and -0 (stored boxes keep the reference's fold
    order) and many equal centroids along the split axis."""
    rng = np.random.default_rng(12)
    v, ip = scenes.triangle_soup(30000, 12, edge=0.01)
    v = v.copy()
    pick = rng.random(v.shape) < 0.2
    v[pick] = np.where(rng.random(pick.sum()) < 0.5, np.float32(0.0), np.float32(-0.0))
    v[:, 0] = np.round(v[:, 0] * 50) / 50  # quantized x: ties in bins and centroids
    _check_static(orc, dev_ctx, v.astype(np.float32), ip, "zeros")


@pytest.mark.gpu
def test_device_build_full_size_soup(orc, dev_ctx):
    """The 1,048,576-triangle benchmark soup."""
    v, ip = scenes.triangle_soup(1 << 20, 2)
    g = _check_static(orc, dev_ctx, v, ip, "1M soup")
    rays = scenes.incoherent_rays(1 << 16, 3)
    h = dev_ctx.trace_mesh(g, rays)
    ref = orc.Mesh(v, ip).trace(rays)
    assert np.array_equal(h["prim"], ref["prim"]) and np.array_equal(h["t"].view(np.uint32), ref["t"].view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("n,seed", [(1, 1), (17, 2), (5000, 3), (40000, 4)])
def test_device_motion_build_matches_oracle(orc, dev_ctx, host_ctx, n, seed):
    v, ip = scenes.motion_soup(n, seed)
    ref = orc.Mesh(v, ip, keys=2).export()
    g = dev_ctx.mesh_build(v, ip, keys=2)
    got = dev_ctx.mesh_export(g)
    assert got["mnodes"].tobytes() == ref["mnodes"].tobytes()
    assert np.array_equal(got["accel_idx"], ref["accel_idx"])
    assert np.array_equal(got["mboxes"].view(np.uint32), ref["mboxes"].view(np.uint32))
    assert np.array_equal(got["idxp"], ref["idxp"])
    # per-key bounds (PolyMesh.motionBounds) as the host builder gives them
    host = host_ctx.mesh_export(host_ctx.mesh_build(v, ip, keys=2))
    assert np.array_equal(got["bounds"].view(np.uint32), host["bounds"].view(np.uint32))


@pytest.mark.gpu
def test_device_build_three_keys(orc, dev_ctx):
    """Three motion keys: the build geometry is key 1 (time 0.5)."""
    rng = np.random.default_rng(4)
    v0, ip = scenes.triangle_soup(3000, 41, edge=0.01)
    v = np.concatenate([v0, v0 + rng.normal(0, 0.02, v0.shape), v0 + rng.normal(0, 0.04, v0.shape)]).astype(np.float32)
    ref = orc.Mesh(v, ip, keys=3).export()
    got = dev_ctx.mesh_export(dev_ctx.mesh_build(v, ip, keys=3))
    assert got["mnodes"].tobytes() == ref["mnodes"].tobytes()
    assert np.array_equal(got["mboxes"].view(np.uint32), ref["mboxes"].view(np.uint32))
    assert np.array_equal(got["accel_idx"], ref["accel_idx"])


@pytest.mark.gpu
def test_device_build_declines_non_finite(dev_ctx):
    v, ip = scenes.triangle_soup(100, 1)
    v = v.copy()
    v[7, 1] = np.inf
    with pytest.raises(vg.VmrError) as e:
        dev_ctx.mesh_build(v, ip)
    assert e.value.code == -7
