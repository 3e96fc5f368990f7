"""Decomposed transforms and the geoms that use them: camera motion keys
(builtin/camera/camera.go:207-236), PolyMesh transform keys
(builtin/geom/polymesh/trace.go:33-48), GeomInstance
(builtin/geom/instance/instance.go) and Proc (builtin/geom/proc/proc.go),
plus DebugShader (builtin/shader/debug.go).

The reference's own tests for math/animdecomp.go and math/matrix4.go print
results without expected values, so the restatement is pinned by a
hand-derived known answer (the polar iteration's one-sided convergence test,
Matrix4Eq at math/matrix4.go:326-336), by properties (rigid keys round trip
to within a few ulp; blending reproduces the end keys) and by agreement of
libvmr's host restatement with the oracle's, bit for bit.  GPU tests compare
scene traces (every hit field) and reference-mode renders with the oracle.
"""
import numpy as np
import pytest

import vermeer_gb300 as vg
from vermeer_gb300 import scenes
from vermeer_gb300.scenes import xf_matrix

from conftest import assert_hits_equal


def _random_keys(rng, n):
    keys = []
    for _ in range(n):
        if rng.random() < 0.5:  # rotation times an axis stretch
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            A = q * rng.uniform(0.3, 2.0, 3)
        else:  # a general matrix
            A = rng.normal(size=(3, 3)) * rng.uniform(0.2, 3.0)
        M = np.eye(4)
        M[:3, :3] = A
        M[:3, 3] = rng.normal(size=3)
        keys.append(M.T.reshape(16).astype(np.float32))
    return np.stack(keys)


# ------------------------------------------------------------------ CPU ----
def test_libvmr_decomposition_equals_oracle(orc):
    rng = np.random.default_rng(3)
    for trial in range(400):
        keys = _random_keys(rng, int(rng.integers(1, 5)))
        t = float(np.float32(rng.random()))
        for blend in (False, True):
            got = vg.transform_keys_at(keys, t, blend)
            ref = orc.keyed_matrix(keys, t, blend)
            assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (trial, blend, got, ref)


def test_polar_iteration_stops_on_the_one_sided_test(orc):
    """diag(2, 0.5, 1): the iteration Q <- (Q + Q^-T)/2 gives diag(1.25,
    1.25, 1), where the 0.5 entry grew by 0.75 > 1e-6, then diag(1.025,
    1.025, 1), where every entry shrank; Matrix4Eq only tests A - B > eps, so
    the reference stops there with Q = diag(1.025, 1.025, 1) instead of the
    identity.  The stretch is Q^T M = diag(2.05, 0.5125, 1), the quaternion
    of Q normalises to the identity, and the rebuilt matrix is that
    stretch (all in float32)."""
    f = np.float32
    q = f((f(1.25) + f(1.0) / f(1.25)) * f(0.5))
    expect = np.eye(4, dtype=np.float32)
    expect[0, 0] = q * f(2.0)
    expect[1, 1] = q * f(0.5)
    m = np.diag([2.0, 0.5, 1.0, 1.0]).astype(np.float32).T.reshape(16)
    T, R, S = orc.decompose(m)
    assert np.array_equal(R, np.float32([0, 0, 0, 1]) * R[3]) and R[3] > 0
    assert S[0] == expect[0, 0] and S[5] == expect[1, 1] and S[10] == 1.0
    for got in (orc.keyed_matrix([m], 0.0), vg.transform_keys_at([m], 0.0)):
        assert np.array_equal(got, expect.T.reshape(16)), got


def test_rigid_keys_round_trip_within_a_few_ulp(orc):
    """A rotation plus translation is its own polar factor after one step;
    rebuilding it from the quaternion changes each element by at most a few
    float32 ulp of 1 (bound 8 ulp = 9.5e-7 on the 3x3 part; 5.5 ulp seen
    over 3000 random rotations).  The translation is
    scaled by the stretch's last diagonal element, which is 1 only to
    rounding (the inverse's corner is a 3x3 cofactor over the 4x4
    determinant): bound 5e-7 relative."""
    rng = np.random.default_rng(5)
    for _ in range(300):
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        if np.linalg.det(q) < 0:
            q[:, 0] = -q[:, 0]
        M = np.eye(4)
        M[:3, :3] = q
        M[:3, 3] = rng.normal(size=3) * 3
        m = M.T.reshape(16).astype(np.float32)
        got = orc.keyed_matrix([m], 0.0).reshape(4, 4).T
        A = m.reshape(4, 4).T
        assert np.abs(got[:3, :3] - A[:3, :3]).max() <= 8 * 2.0 ** -23
        assert np.all(np.abs(got[:3, 3] - A[:3, 3]) <= 5e-7 * np.abs(A[:3, 3]) + 1e-30)


def test_blending_reproduces_the_end_keys(orc):
    """TransformDecompLerp at t = 0 and t = 1 of two keys gives each key's
    own rebuilt matrix (the slerp returns an end quaternion there)."""
    rng = np.random.default_rng(7)
    for _ in range(100):
        keys = _random_keys(rng, 2)
        k0 = orc.keyed_matrix(keys[:1], 0.0)
        k1 = orc.keyed_matrix(keys[1:], 0.0)
        assert np.array_equal(orc.keyed_matrix(keys, 0.0), k0)
        assert np.array_equal(orc.keyed_matrix(keys, 1.0), k1)


def test_capi_validates_groups(host_ctx):
    v, ip = scenes.triangle_soup(50, 3)
    g = host_ctx.mesh_build(v, ip)
    k = [xf_matrix(0.3, (0, 1, 0), (1, 1, 1), (0, 0, 0))]
    inst = host_ctx.instance_add(g, k, (-1, -1, -1), (1, 1, 1))
    with pytest.raises(vg.VmrError) as e:
        host_ctx.instance_add(inst, k, (-1, -1, -1), (1, 1, 1))
    assert e.value.code == -7  # VMR_ERR_UNSUPPORTED: instance of an instance
    c = host_ctx.mesh_build(v, ip)
    # (distinct box centres: equal centroids make the reference's top-level
    # split recurse forever, qbvh/build.go:34-43)
    proc = host_ctx.proc_add([c], None, (-1, -1, -1), (2, 2, 2))
    with pytest.raises(vg.VmrError):
        host_ctx.scene_build([g, c])  # a Proc's child joins no scene itself
    with pytest.raises(vg.VmrError):
        host_ctx.proc_add([c], None, (-1, -1, -1), (1, 1, 1))  # one Proc per child
    host_ctx.scene_build([g, inst, proc])


def test_oracle_instance_matches_pretransformed_mesh(orc):
    """An instance with one key sees its geom where the rebuilt matrix puts
    it: hits at the distances of a mesh built from vertices moved by that
    matrix (to float32 rounding of the two routes)."""
    v, ip = scenes.triangle_soup(30000, 71, lo=-0.5, hi=0.5, edge=0.02)
    k = xf_matrix(0.6, (1, 2, 3), (1.1, 0.9, 1.0), (0.1, 0.0, -0.1))
    base = orc.Mesh(v, ip)
    inst = orc.Instance(base, [k], (-2, -2, -2), (2, 2, 2))
    sc = orc.Scene([inst])
    A = orc.keyed_matrix([k], 0.0).reshape(4, 4).T.astype(np.float64)
    pre = orc.Mesh((v.reshape(-1, 3).astype(np.float64) @ A[:3, :3].T + A[:3, 3]).astype(np.float32), ip)
    rays = scenes.incoherent_rays(20000, 72, lo=-1.0, hi=1.0)
    got, ref = sc.trace(rays), orc.Scene([pre]).trace(rays)
    both = (got["prim"] >= 0) & (ref["prim"] >= 0)
    assert both.sum() > 3000
    assert (got["prim"] >= 0).sum() == pytest.approx((ref["prim"] >= 0).sum(), rel=0.01)
    assert np.allclose(got["t"][both], ref["t"][both], rtol=1e-4, atol=1e-5)


# ------------------------------------------------------------------ GPU ----
W = H = 64
ITERS = 4


@pytest.mark.gpu
@pytest.mark.parametrize("tuning", [(45, 0, 0, 0, 8), (0, 0, 0, 0, 0)])
def test_scene_with_instances_procs_and_keys_matches_oracle(ctx, orc, tuning):
    sc = scenes.small_room_groups(2048, seed=4)
    ids = ctx.load_scene(sc)
    geoms = orc.build_geoms(sc["meshes"])
    osc = orc.scene_of(sc["meshes"], geoms)
    rays = scenes.incoherent_rays(120000, 95, lo=-0.95, hi=0.95)
    rays[:, 7] = scenes.uniform(96, rays.shape[0], 1).astype(np.float32)
    idmap = np.asarray(ids, np.int32)
    try:
        ctx.set_tuning(*tuning)
        for shadow in (False, True):
            got = ctx.trace_scene(rays, shadow=shadow)
            ref = osc.trace(rays, shadow=shadow)
            ref["geom"] = np.where(ref["geom"] >= 0, idmap[np.maximum(ref["geom"], 0)], -1)
            assert_hits_equal(got, ref, keys=("prim", "geom", "t", "u", "v", "w"),
                              what=f"groups tuning={tuning} shadow={shadow}")
        hit_ids = set(np.unique(got["geom"]).tolist())
        n0 = len(scenes.small_room(2048, seed=4)["meshes"])
        assert {ids[n0 + 1], ids[n0 + 2], ids[n0 + 4]} <= hit_ids   # the instances
        assert {ids[n0 + 5], ids[n0 + 6]} & hit_ids                   # a Proc's children
    finally:
        ctx.set_tuning(45, 0, 0, 0, 8)


def _compare(got, ref):
    assert not np.isnan(got).any() and not np.isnan(ref).any()
    ok = np.abs(got - ref) <= 1e-5 * (1.0 + np.abs(ref))
    return ok.all(-1).mean(), np.abs(got - ref).mean()


@pytest.mark.gpu
@pytest.mark.parametrize("camera_keys", [False, True])
def test_render_with_groups_keys_and_debug_shader_matches_oracle(ctx, orc, camera_keys):
    """Reference-mode render of the room with instances, a Proc, keyed mesh
    transforms, a DebugShader and (camera_keys) camera motion keys."""
    sc = scenes.small_room_groups(2048, seed=4, camera_keys=camera_keys)
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(W, H, 0, ITERS, 11)
    got, st = ctx.render(W, H, 0, ITERS, 11)
    frac, mean_abs = _compare(got, ref)
    assert frac >= 0.999, (frac, mean_abs)
    assert mean_abs <= 1e-6, (frac, mean_abs)
    # the DebugShader's colour shows up unlit on the back wall, folded as
    # core.Render folds a constant c: buf = (buf*j + c)/(j+1) from j = 1 on
    # a zero buffer gives c*N/(N+1) after N iterations (core/render.go:127-129)
    dbg = np.float32([0.9, 0.2, 0.6]) * np.float32(ITERS) / np.float32(ITERS + 1)
    assert (np.abs(got - dbg).max(-1) < 1e-6).mean() > 0.05


@pytest.mark.gpu
def test_one_key_camera_uses_the_rebuilt_matrix(ctx, orc):
    """vmr_set_camera renders with the matrix rebuilt from the camera's
    decomposition, as the reference does: for a camera matrix with a stretch
    the image differs from one made with the raw matrix, and it equals the
    oracle's (which rebuilds the same way)."""
    sc = scenes.small_room(2048, seed=6)
    cam = sc["camera"]
    m = np.asarray(cam["m"], np.float32).copy()
    m[0:3] *= np.float32(1.3)  # stretch the camera's x axis
    cam["m"] = m
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(W, H, 0, 2, 3)
    got, _ = ctx.render(W, H, 0, 2, 3)
    frac, mean_abs = _compare(got, ref)
    assert frac >= 0.999 and mean_abs <= 1e-6, (frac, mean_abs)
    rebuilt = orc.keyed_matrix([m], 0.0, True)
    assert not np.array_equal(rebuilt, m)


@pytest.mark.gpu
@pytest.mark.parametrize("camera_keys", [False, True])
def test_path_tracer_with_groups_matches_float_oracle(ctx, orc, camera_keys):
    """The extended mode over the room with instances (one key and two), an
    instanced sphere, a Proc with a transformed child, a mesh with transform
    keys and (camera_keys) camera keys: the traversal takes the single-loop
    scene kernel and the shading applies each hit's group or keyed
    transform at the ray's time, as the float oracle does."""
    sc = dict(scenes.small_room_groups(2048, seed=4, camera_keys=camera_keys, debug=False), env=(0.1, 0.1, 0.12))
    ctx.load_scene(sc)
    ref, _ = orc.Render(sc).run_path(40, 40, 0, 3, 23, max_depth=4, precision=32)
    got, _ = ctx.render_path(40, 40, 0, 3, 23, max_depth=4)
    ok = (np.abs(got - ref) <= 1e-5 * (1 + np.abs(ref))).all(-1)
    assert ok.mean() >= 0.999, ok.mean()
    assert abs(got.mean() - ref.mean()) <= 1e-4 * ref.mean()


@pytest.mark.gpu
def test_path_tracer_refuses_debug_shader_and_grouped_jobs(ctx):
    """A DebugShader renders in reference mode only; batched path jobs take
    plain meshes (an instance as a job is refused)."""
    sc = scenes.small_room_groups(1024, seed=4, camera_keys=False)
    ids = ctx.load_scene(sc)
    with pytest.raises(vg.VmrError) as e:
        ctx.render_path(16, 16, 0, 1, 1)
    assert e.value.code == -7
    inst = next(ids[i] for i, m in enumerate(sc["meshes"]) if "instance" in m)
    with pytest.raises(vg.VmrError) as e:
        ctx.render_path_jobs([dict(geom=inst, width=16, height=16, camera=sc["camera"])], 0, 1, 1, max_depth=2)
    assert e.value.code == -7
