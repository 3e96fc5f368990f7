"""Normals of motion meshes: PolyMesh.Normals with as many motion keys as
the vertices.  TraceMotionElems (builtin/geom/polymesh/trace.go:694-712)
reads corner j of the hit element idx at Normals.Elems[idx*3 + j +
ElemsPerKey*key] (directly, not through NormalIdx), lerps the two keys
around the ray's time, weights the corners by the hit's barycentrics and
normalises; without such normals N = Ng.

CPU tests: the oracle uses the normals (the image changes) and refuses
short or mis-keyed arrays, libvmr refuses them the same way before any
device work, and a .vnf PolyMesh with keyed Normals loads.  GPU tests: the
reference-mode and extended-mode renders equal the oracle's in both
motion leaf-indexing modes, and the .vnf scene renders as the scene built
directly.
"""
import numpy as np
import pytest

from vermeer_gb300 import scenes

INVALID = -1
REL, FRAC_EQUAL, MEAN_ABS = 1e-5, 0.999, 1e-6


def _compare(got, ref):
    assert not np.isnan(got).any() and not np.isnan(ref).any()
    ok = (np.abs(got - ref) <= REL * (1.0 + np.abs(ref))).all(-1)
    return ok.mean(), np.abs(got - ref).mean()


# ------------------------------------------------------------------ CPU ----
def test_oracle_motion_normals_shade(orc):
    """The keyed corner normals reach the shading: same traversal, another
    image; without them N = Ng as before."""
    plain = scenes.small_room_motion(1024, seed=9)
    withn = scenes.small_room_motion(1024, seed=9, normals=True)
    a = orc.Render(plain).run(32, 32, 0, 2, 5)
    b = orc.Render(withn).run(32, 32, 0, 2, 5)
    assert np.isfinite(b).all() and (b >= 0).all()
    assert np.abs(a - b).max() > 1e-3


def test_oracle_motion_normals_validation(orc):
    sc = scenes.small_room_motion(256, seed=9, normals=True)
    soup = sc["meshes"][1]
    m = orc.Mesh(soup["verts"], soup["idxp"], keys=2)
    mn = soup["motion_normals"]
    m.set_motion_normals(mn)
    with pytest.raises(ValueError):
        m.set_motion_normals(mn[:1])  # one key for a two-key mesh
    with pytest.raises(ValueError):
        m.set_motion_normals(mn[:, :-1])  # fewer than 3 per triangle
    s = orc.Mesh(soup["verts"][: soup["verts"].shape[0] // 2], soup["idxp"])
    with pytest.raises(ValueError):
        s.set_motion_normals(mn)  # a static mesh


def test_capi_motion_normals_refused_before_device_work(host_ctx):
    import ctypes
    sc = scenes.small_room_motion(256, seed=9, normals=True)
    soup = sc["meshes"][1]
    mn = np.ascontiguousarray(soup["motion_normals"])
    g = host_ctx.mesh_build(soup["verts"], soup["idxp"], keys=2)
    s = host_ctx.mesh_build(soup["verts"][: soup["verts"].shape[0] // 2], soup["idxp"])
    L, P = host_ctx.L, ctypes.c_void_p
    ptr = P(mn.ctypes.data)
    n = mn.shape[1]
    assert L.vmr_mesh_set_motion_normals(host_ctx.h, g, ptr, n, 2) == 0
    assert L.vmr_mesh_set_motion_normals(host_ctx.h, g, ptr, n, 3) == INVALID
    assert L.vmr_mesh_set_motion_normals(host_ctx.h, g, ptr, n - 1, 2) == INVALID
    assert L.vmr_mesh_set_motion_normals(host_ctx.h, s, ptr, n, 2) == INVALID
    assert L.vmr_mesh_set_motion_normals(host_ctx.h, g, None, 0, 0) == 0


def test_vnf_motion_normals_load(host_ctx, tmp_path):
    """A motion PolyMesh whose Normals have as many keys as its Verts loads
    (it was refused before the keyed normals were supported)."""
    sc = scenes.small_room_motion(256, seed=9, normals=True)
    path = tmp_path / "mn.vnf"
    path.write_text(scenes.to_vnf(sc, 32, 32))
    info = host_ctx.load_vnf(str(path))
    assert info["n_geoms"] == len(sc["meshes"])


# ------------------------------------------------------------------ GPU ----
@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1])
def test_render_motion_normals_match_oracle(ctx, orc, mode):
    sc = scenes.small_room_motion(2048, seed=9, motion_mode=mode, normals=True)
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(48, 48, 0, 3, 19)
    got, _ = ctx.render(48, 48, 0, 3, 19)
    frac, mean_abs = _compare(got, ref)
    assert frac >= FRAC_EQUAL and mean_abs <= MEAN_ABS, (frac, mean_abs)
    # the normals are in use: the image differs from the one without them
    plain = scenes.small_room_motion(2048, seed=9, motion_mode=mode)
    ctx.load_scene(plain)
    other, _ = ctx.render(48, 48, 0, 3, 19)
    assert np.abs(other - got).max() > 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1])
def test_pt_motion_normals_match_float_oracle(ctx, orc, mode):
    sc = dict(scenes.small_room_motion(2048, seed=12, motion_mode=mode, normals=True), env=(0.1, 0.1, 0.12))
    ctx.load_scene(sc)
    ref, _ = orc.Render(sc).run_path(40, 40, 0, 3, 23, max_depth=4, precision=32)
    got, _ = ctx.render_path(40, 40, 0, 3, 23, max_depth=4)
    ok = (np.abs(got - ref) <= REL * (1 + np.abs(ref))).all(-1)
    assert ok.mean() >= FRAC_EQUAL, ok.mean()
    assert abs(got.mean() - ref.mean()) <= 1e-4 * ref.mean()


@pytest.mark.gpu
def test_vnf_motion_normals_render_equals_direct_scene(ctx, tmp_path):
    sc = scenes.small_room_motion(1024, seed=6, normals=True)
    path = tmp_path / "mn.vnf"
    path.write_text(scenes.to_vnf(sc, 40, 30))
    ctx.load_scene(scenes.vnf_order(sc))
    ref, _ = ctx.render(40, 30, 0, 3, 5)
    info = ctx.load_vnf(str(path))
    got, _ = ctx.render(info["width"], info["height"], 0, 3, 5)
    assert got.tobytes() == ref.tobytes()
