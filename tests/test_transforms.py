"""Per-mesh transforms (PolyMesh.Transform with one matrix,
builtin/geom/polymesh/trace.go:15-101): a scene trace that enters the mesh
walks it with the ray mapped into object space by Matrix4Inverse of the
matrix and Ray.Setup, then continues with the world ray; the top level keeps
the mesh's object-space bounds, as PolyMesh.Bounds does.

CPU tests check the oracle's semantics against meshes whose vertices are
transformed beforehand, and the C ABI's validation; GPU tests compare scene
traces (closest and any hit, static and motion meshes, three kernels) and
both render modes with the oracle.
"""
import numpy as np
import pytest

from vermeer_gb300 import scenes

from conftest import assert_hits_equal


def _matrix(angle, axis, scale, centre, shift):
    """Column-major 4x4 (math.Matrix4 order) of x -> centre + shift + R S (x - centre)."""
    axis = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K
    A = np.eye(4)
    A[:3, :3] = R @ np.diag(scale)
    c = np.asarray(centre, np.float64)
    A[:3, 3] = c + np.asarray(shift) - A[:3, :3] @ c
    return A.T.reshape(16).astype(np.float32)


def _apply(m16, v):
    A = m16.reshape(4, 4).T.astype(np.float64)
    return (v.astype(np.float64) @ A[:3, :3].T + A[:3, 3]).astype(np.float32)


def _scene(rng, n_meshes=16, motion_every=0):
    ms, xfs = [], []
    for i in range(n_meshes):
        n = int(rng.integers(200, 4000))
        if motion_every and i % motion_every == 1:
            v, ip = scenes.motion_soup(n, 800 + i, edge=0.01)
            k = 2
        else:
            v, ip = scenes.triangle_soup(n, 800 + i, edge=0.01)
            k = 1
        off = rng.uniform(-1, 1, 3).astype(np.float32)
        v = (v * 0.6 + off).astype(np.float32)
        xf = None
        if i % 3 != 2:  # most meshes transformed: a turn about their centre, a stretch, a small shift
            c = v.reshape(-1, 3).mean(0)
            xf = _matrix(rng.uniform(0.2, 0.9), rng.normal(size=3), rng.uniform(0.8, 1.2, 3), c,
                         rng.uniform(-0.05, 0.05, 3))
        ms.append((v, ip, k))
        xfs.append(xf)
    return ms, xfs


def test_oracle_transform_matches_pretransformed_vertices(orc):
    """Rays that cross the mesh's object-space box see the transformed mesh:
    the hits of a mesh built from transformed vertices, at the same
    distances to float32 rounding; rays that only cross the
    transformed copy see nothing (the top level boxes the untransformed
    mesh, as the reference's does)."""
    v, ip = scenes.triangle_soup(3000, 71, edge=0.02)
    xf = _matrix(0.6, (1, 2, 3), (1.1, 0.9, 1.0), v.reshape(-1, 3).mean(0), (0.02, 0.0, -0.01))
    om = orc.Mesh(v, ip)
    om.set_transform(xf)
    sc = orc.Scene([om])
    pre = orc.Mesh(_apply(xf, v.reshape(-1, 3)).reshape(v.shape), ip)
    sc_pre = orc.Scene([pre])
    rays = scenes.incoherent_rays(20000, 72)
    got, ref = sc.trace(rays), sc_pre.trace(rays)
    # a ray whose hit on the transformed copy lies inside the object-space
    # box crosses that box, so it enters the mesh and finds the same triangle
    P = rays[:, :3] + ref["t"][:, None] * rays[:, 3:6]
    lo, hi = v.reshape(-1, 3).min(0), v.reshape(-1, 3).max(0)
    inside = (ref["prim"] >= 0) & np.all((P > lo) & (P < hi), axis=1)
    assert inside.sum() > 2000
    # (static ElemIDs are leaf-order positions, which differ between the two
    # builds: compare hits and distances)
    both = inside & (got["prim"] >= 0)
    assert both.sum() > 0.99 * inside.sum(), (both.sum(), inside.sum())
    close = np.abs(got["t"][both] - ref["t"][both]) <= 1e-4 * ref["t"][both] + 1e-5
    assert close.mean() > 0.99, close.mean()
    # far away the object box is missed: translated copies are invisible there
    far = _matrix(0.0, (0, 0, 1), (1, 1, 1), (0, 0, 0), (5.0, 0.0, 0.0))
    om2 = orc.Mesh(v, ip)
    om2.set_transform(far)
    r2 = scenes.incoherent_rays(5000, 73, lo=4.8, hi=5.2)
    assert (orc.Scene([om2]).trace(r2)["prim"] < 0).all()


def test_transform_validation(host_ctx):
    import vermeer_gb300 as vg
    v, ip = scenes.triangle_soup(10, 74, edge=0.05)
    g = host_ctx.mesh_build(v, ip)
    host_ctx.mesh_set_transform(g, np.eye(4, dtype=np.float32).reshape(16))
    host_ctx.mesh_set_transform(g, None)
    with pytest.raises(vg.VmrError):
        host_ctx.mesh_set_transform(g + 100, np.eye(4, dtype=np.float32).reshape(16))
    s = host_ctx.sphere_add((0, 0, 0), 1.0)
    with pytest.raises(vg.VmrError):
        host_ctx.mesh_set_transform(s, np.eye(4, dtype=np.float32).reshape(16))


# ------------------------------------------------------------------ GPU ----
@pytest.mark.gpu
@pytest.mark.parametrize("motion_every,tuning", [(0, (45, 0, 0, 0, 8)), (0, (13, 0, 0, 0, 4)), (0, (0, 0, 0, 0, 0)),
                                                 (3, (45, 0, 0, 0, 8)), (3, (0, 0, 0, 0, 0))])
def test_scene_with_transforms_matches_oracle(ctx, orc, motion_every, tuning):
    rng = np.random.default_rng(81 + motion_every)
    ms, xfs = _scene(rng, motion_every=motion_every)
    oms, ids = [], []
    for (v, ip, k), xf in zip(ms, xfs):
        om = orc.Mesh(v, ip, keys=k, motion_fixed=True)
        g = ctx.mesh_build(v, ip, keys=k, motion_mode=1)
        if xf is not None:
            om.set_transform(xf)
            ctx.mesh_set_transform(g, xf)
        oms.append(om)
        ids.append(g)
    osc = orc.Scene(oms)
    ctx.scene_build(ids)
    rays = np.concatenate([scenes.incoherent_rays(80000, 82, lo=-1.5, hi=1.5),
                           scenes.coherent_rays(200, eye=(0.0, 0.0, -3.0), target=(0.0, 0.0, 0.0))])
    rays[:, 7] = scenes.uniform(83, rays.shape[0], 3).astype(np.float32)
    try:
        ctx.set_tuning(*tuning)
        for shadow in (False, True):
            got = ctx.trace_scene(rays, shadow=shadow)
            ref = osc.trace(rays, shadow=shadow)
            ref["geom"] = np.where(ref["geom"] >= 0, np.asarray(ids, np.int32)[np.maximum(ref["geom"], 0)], -1)
            if shadow:
                assert np.array_equal(got["prim"] >= 0, ref["prim"] >= 0)
            else:
                assert_hits_equal(got, ref, keys=("prim", "geom", "t", "u", "v", "w"),
                                  what=f"transforms tuning={tuning}")
                xf_ids = np.asarray([g for g, xf in zip(ids, xfs) if xf is not None])
                assert np.isin(got["geom"][got["prim"] >= 0], xf_ids).sum() > 1000
    finally:
        ctx.set_tuning(45, 0, 0, 0, 8)


def _transformed_room(kind):
    sc = scenes.small_room(2048, seed=6) if kind == "reference" else scenes.small_room_ext(2048, seed=6)
    sc = dict(sc, meshes=[dict(m) for m in sc["meshes"]])
    for m in sc["meshes"]:
        if "sphere" in m or m.get("keys", 1) > 1 or len(m["idxp"]) < 300:
            continue  # the soup: turned about the room's centre and stretched
        m["transform"] = _matrix(0.35, (0.3, 1.0, 0.2), (1.05, 0.95, 1.0), (0.0, 0.0, 0.0), (0.0, 0.03, 0.0))
    assert any("transform" in m for m in sc["meshes"])
    return sc


@pytest.mark.gpu
def test_reference_render_with_transform_matches_oracle(ctx, orc):
    """core.Render over a room whose soup is transformed: hit points and
    normals go to world space as core.Trace's ApplyTransform does."""
    sc = _transformed_room("reference")
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(48, 40, 0, 2, 5)
    got, _ = ctx.render(48, 40, 0, 2, 5)
    ok = np.abs(got - ref) <= 1e-5 * (1.0 + np.abs(ref))
    assert ok.all(-1).mean() >= 0.999, ok.all(-1).mean()
    base = orc.Render(dict(sc, meshes=[{k: v for k, v in m.items() if k != "transform"} for m in sc["meshes"]]))
    assert not np.array_equal(base.run(48, 40, 0, 2, 5), ref)  # the transform changes the image


@pytest.mark.gpu
def test_path_render_with_transform_matches_float_oracle(ctx, orc):
    sc = _transformed_room("extended")
    ctx.load_scene(sc)
    ref, _ = orc.Render(sc).run_path(40, 32, 0, 3, 9, max_depth=4, precision=32)
    got, _ = ctx.render_path(40, 32, 0, 3, 9, max_depth=4)
    ok = (np.abs(got - ref) <= 1e-5 * (1 + np.abs(ref))).all(-1)
    assert ok.mean() >= 0.995, ok.mean()


@pytest.mark.gpu
def test_path_jobs_with_a_transformed_mesh_equal_one_scene_renders(ctx):
    """A job whose mesh has a transform renders as that mesh alone in a
    scene does (the job-mode entry maps the ray as the top-level leaf
    would), static and motion meshes, bit for bit."""
    bj = scenes.batched_jobs(n_jobs=4, seed=11, width=32, height=24, lo=800, hi=3000)
    ids = []
    for k, m in enumerate(bj["meshes"]):
        g = ctx.mesh_build(m["verts"], m["idxp"], keys=m.get("keys", 1), motion_mode=m.get("motion_mode", 0))
        if k < 2:  # one static and one motion job transformed
            c = np.asarray(m["verts"], np.float32).reshape(-1, 3).mean(0)
            ctx.mesh_set_transform(g, _matrix(0.4, (1, 1, 0), (1.1, 0.9, 1.0), c, (0.0, 0.01, 0.0)))
        ids.append(g)
    ctx.set_shaders(bj["shaders"])
    for g in ids:
        ctx.mesh_set_shading(g, [0])
    ctx.set_lights([])
    ctx.set_quad_lights([])
    ctx.set_env_light(bj["env"])
    jobs = [dict(geom=g, width=32, height=24, camera=bj["cameras"][k]) for k, g in enumerate(ids)]
    imgs, _ = ctx.render_path_jobs(jobs, 0, 2, 17, max_depth=4)
    for k, g in enumerate(ids):
        ctx.scene_build([g])
        ctx.set_camera(bj["cameras"][k])
        ref, _ = ctx.render_path(32, 24, 0, 2, 17, max_depth=4)
        assert imgs[k].tobytes() == ref.tobytes(), k
