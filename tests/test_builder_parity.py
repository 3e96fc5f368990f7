"""The product's host QBVH builder (libvmr, vmr_mesh_build / vmr_scene_build)
produces node arrays identical to the oracle's restatement of the reference
builder (qbvh/build.go, builtin/geom/polymesh/buildqbvh.go,
builtin/scene/scene.go).  Runs on a host-only context: no GPU needed."""
import numpy as np
import pytest

from vermeer_gb300 import scenes


def _same_nodes(a, b):
    assert a.shape == b.shape, (a.shape, b.shape)
    assert a.tobytes() == b.tobytes()


def _soups():
    yield "one", *scenes.triangle_soup(1, 1)
    yield "sixteen", *scenes.triangle_soup(16, 2)
    yield "seventeen", *scenes.triangle_soup(17, 3)
    yield "small", *scenes.triangle_soup(1000, 4)
    yield "medium", *scenes.triangle_soup(60000, 5, edge=0.01)
    # degenerate: every centroid identical (flat centroid bounds, build.go:34-43)
    v, ip = scenes.triangle_soup(40, 6)
    t = v.reshape(-1, 3, 3)
    t[:] = t[0]
    yield "identical", t.reshape(-1, 3), ip
    # planar: all triangles in z = 0.5
    v, ip = scenes.triangle_soup(3000, 7, edge=0.02)
    v[:, 2] = 0.5
    yield "planar", v, ip
    # shared vertices (an indexed mesh): a 40x40 grid of quads
    n = 40
    g = np.stack(np.meshgrid(np.linspace(0, 1, n + 1), np.linspace(0, 1, n + 1), indexing="ij"), -1).reshape(-1, 2)
    verts = np.concatenate([g, 0.3 * np.sin(7 * g[:, :1])], 1).astype(np.float32)
    idx = []
    for i in range(n):
        for j in range(n):
            a, b, c, d = i * (n + 1) + j, (i + 1) * (n + 1) + j, (i + 1) * (n + 1) + j + 1, i * (n + 1) + j + 1
            idx += [a, b, c, a, c, d]
    yield "grid", verts, np.asarray(idx, np.uint32)


@pytest.mark.parametrize("case", list(range(8)))
def test_static_mesh_build_matches_oracle(orc, host_ctx, case):
    name, v, ip = list(_soups())[case]
    ref = orc.Mesh(v, ip).export()
    g = host_ctx.mesh_build(v, ip)
    got = host_ctx.mesh_export(g)
    _same_nodes(got["nodes"], ref["nodes"])
    assert np.array_equal(got["accel_idx"], ref["accel_idx"]), name
    assert np.array_equal(got["idxp"], ref["idxp"]), name
    assert np.array_equal(got["bounds"].view(np.uint32), ref["bounds"].view(np.uint32)), name


@pytest.mark.parametrize("n,seed", [(1, 1), (17, 2), (5000, 3), (40000, 4)])
def test_motion_mesh_build_matches_oracle(orc, host_ctx, n, seed):
    v, ip = scenes.motion_soup(n, seed)
    om = orc.Mesh(v, ip, keys=2)
    ref = om.export()
    g = host_ctx.mesh_build(v, ip, keys=2)
    got = host_ctx.mesh_export(g)
    _same_nodes(got["mnodes"], ref["mnodes"])
    assert np.array_equal(got["accel_idx"], ref["accel_idx"])
    assert np.array_equal(got["mboxes"].view(np.uint32), ref["mboxes"].view(np.uint32))
    assert np.array_equal(got["idxp"], ref["idxp"])


def _scene_meshes(seed, n_meshes, motion_every=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_meshes):
        n = int(rng.integers(1, 400))
        if motion_every and i % motion_every == 0:
            v, ip = scenes.motion_soup(n, seed * 100 + i)
            keys = 2
        else:
            v, ip = scenes.triangle_soup(n, seed * 100 + i)
            keys = 1
        off = rng.uniform(-2, 2, 3).astype(np.float32)
        out.append(((v + off).astype(np.float32), ip, keys))
    return out


@pytest.mark.parametrize("seed,n_meshes,motion_every", [(1, 1, 0), (2, 7, 0), (3, 40, 0), (4, 9, 2), (5, 30, 3)])
def test_scene_top_level_matches_oracle(orc, host_ctx, seed, n_meshes, motion_every):
    ms = _scene_meshes(seed, n_meshes, motion_every)
    oms = [orc.Mesh(v, ip, keys=k) for v, ip, k in ms]
    ref = orc.Scene(oms).export()
    ids = [host_ctx.mesh_build(v, ip, keys=k) for v, ip, k in ms]
    host_ctx.scene_build(ids)
    got = host_ctx.scene_export(len(ids))
    assert got["keys"] == ref["keys"]
    assert np.array_equal(got["geom_order"], np.asarray(ids, np.uint32)[ref["geom_order"]])
    _same_nodes(got["nodes"], ref["nodes"])
    _same_nodes(got["mnodes"], ref["mnodes"])
    assert np.array_equal(got["mboxes"].view(np.uint32), ref["mboxes"].view(np.uint32))


def test_builder_rejects_bad_input(host_ctx):
    import vermeer_gb300 as vg
    v, ip = scenes.triangle_soup(10, 1)
    bad = ip.copy()
    bad[5] = 10**6
    with pytest.raises(vg.VmrError) as e:
        host_ctx.mesh_build(v, bad)
    assert e.value.code == -1
