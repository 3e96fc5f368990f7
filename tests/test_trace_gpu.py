"""Bit-exact parity of the CUDA traversal (through the C ABI) with the CPU
oracle: closest-hit and any-hit, static, motion (faithful and fixed) and
two-level scenes, host and device buffers, golden fixtures and the full
1M-triangle / 4M-ray workload."""
import os

import numpy as np
import pytest

from conftest import assert_hits_equal
from vermeer_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_golden_fixture_static(ctx):
    g = np.load(os.path.join(GOLDEN, "traversal_small.npz"))
    for case in ("soup64", "soup2k", "soup8k"):
        geom = ctx.mesh_build(g[f"{case}__verts"], g[f"{case}__idxp"])
        rays = g[f"{case}__rays"]
        for mode, shadow in (("ch", False), ("any", True)):
            got = ctx.trace_mesh(geom, rays, shadow=shadow)
            ref = {k: g[f"{case}__{mode}_{k}"] for k in ("prim", "t", "u", "v", "w")}
            assert_hits_equal(got, ref, what=f"{case}/{mode}")


@pytest.mark.parametrize("n,seed,edge", [(1, 1, 0.3), (17, 2, 0.2), (5000, 3, 0.02), (100000, 4, 0.005)])
def test_static_parity_incoherent(ctx, orc, n, seed, edge):
    v, ip = scenes.triangle_soup(n, seed, edge=edge)
    rays = scenes.incoherent_rays(200000, seed + 50)
    geom = ctx.mesh_build(v, ip)
    om = orc.Mesh(v, ip)
    for shadow in (False, True):
        assert_hits_equal(ctx.trace_mesh(geom, rays, shadow=shadow), om.trace(rays, shadow=shadow),
                          what=f"n={n} shadow={shadow}")


def test_static_parity_coherent_and_finite_tmax(ctx, orc):
    v, ip = scenes.triangle_soup(200000, 8)
    geom = ctx.mesh_build(v, ip)
    om = orc.Mesh(v, ip)
    rays = scenes.coherent_rays(384)
    assert_hits_equal(ctx.trace_mesh(geom, rays), om.trace(rays), what="coherent")
    rays = scenes.incoherent_rays(100000, 9)
    rays[:, 6] = np.random.default_rng(0).uniform(0, 0.05, rays.shape[0]).astype(np.float32)
    for shadow in (False, True):
        assert_hits_equal(ctx.trace_mesh(geom, rays, shadow=shadow), om.trace(rays, shadow=shadow),
                          what=f"finite tmax shadow={shadow}")


def test_uploaded_reference_tree_equals_built(ctx, orc):
    """A reference-built tree uploaded through vmr_mesh_upload traces the
    same as the tree libvmr builds itself."""
    v, ip = scenes.triangle_soup(30000, 10)
    ex = orc.Mesh(v, ip).export()
    g_up = ctx.mesh_upload(v, ex["idxp"], ex["accel_idx"], nodes=ex["nodes"], bounds=ex["bounds"])
    g_b = ctx.mesh_build(v, ip)
    rays = scenes.incoherent_rays(50000, 11)
    assert_hits_equal(ctx.trace_mesh(g_up, rays), ctx.trace_mesh(g_b, rays), what="upload vs build")


def test_device_buffers_equal_host_buffers(ctx):
    import torch
    v, ip = scenes.triangle_soup(50000, 12)
    geom = ctx.mesh_build(v, ip)
    rays = scenes.incoherent_rays(100000, 13)
    host = ctx.trace_mesh(geom, rays)
    dev_rays = torch.from_numpy(np.ascontiguousarray(rays.T)).cuda()
    dev = ctx.trace_mesh(geom, dev_rays)
    ctx.sync()
    got = {k: dev[k].cpu().numpy() for k in ("prim", "t", "u", "v", "w")}
    assert_hits_equal(got, host, what="device vs host")


def test_counters_match_oracle_visit_counts(ctx, orc):
    """The visit counters report the reference's NodesT / LeafsT totals
    (the GPU skips only pops the reference culls)."""
    v, ip = scenes.triangle_soup(20000, 14)
    geom = ctx.mesh_build(v, ip)
    rays = scenes.incoherent_rays(20000, 15)
    got = ctx.trace_mesh(geom, rays, counters=True)["stats"]
    ref = orc.Mesh(v, ip).trace(rays, counters=True)["counters"].astype(np.uint64).sum(axis=0)
    assert got["node_visits"] == ref[0] and got["leaf_visits"] == ref[1] and got["tri_tests"] == ref[2]


@pytest.mark.parametrize("fixed", [False, True])
@pytest.mark.parametrize("n,seed", [(12, 1), (3000, 2), (60000, 3)])
def test_motion_parity(ctx, orc, n, seed, fixed):
    v, ip = scenes.motion_soup(n, seed, edge=0.01)
    rays = scenes.incoherent_rays(100000, seed + 7)
    rays[:, 7] = scenes.uniform(seed, rays.shape[0], 77).astype(np.float32)
    rays[:3, 7] = [0.0, 1.0, 0.5]
    mode = 1 if fixed else 0
    geom = ctx.mesh_build(v, ip, keys=2, motion_mode=mode)
    om = orc.Mesh(v, ip, keys=2, motion_fixed=fixed)
    for shadow in (False, True):
        assert_hits_equal(ctx.trace_mesh(geom, rays, shadow=shadow), om.trace(rays, shadow=shadow),
                          what=f"motion fixed={fixed} shadow={shadow}")


@pytest.mark.parametrize("motion_every,tuning", [(0, (45, 0, 0, 0, 8)), (2, (45, 0, 0, 0, 8)), (2, (45, 0, 0, 0, 0)),
                                                 (2, (13, 0, 0, 0, 4)), (2, (0, 0, 0, 0, 0)), (3, (41, 0, 0, 0, 8))])
def test_two_level_scene_parity(ctx, orc, motion_every, tuning):
    """Two-level scenes, static and with motion meshes (which give the top
    level motion keys): the while-while scene kernel (its motion
    instantiation lerps the top-level and mesh boxes, motion leaves scanned
    per lane) and the single-loop kernel (tuning 0) equal the oracle."""
    ctx.set_tuning(*tuning)
    try:
        _two_level_scene_parity(ctx, orc, motion_every)
    finally:
        ctx.set_tuning(45, 0, 0, 0, 8)


def _two_level_scene_parity(ctx, orc, motion_every):
    rng = np.random.default_rng(5 + motion_every)
    ms = []
    for i in range(24):
        n = int(rng.integers(1, 5000))
        if motion_every and i % motion_every == 0:
            v, ip = scenes.motion_soup(n, 500 + i, edge=0.01)
            k = 2
        else:
            v, ip = scenes.triangle_soup(n, 500 + i, edge=0.01)
            k = 1
        off = rng.uniform(-1, 1, 3).astype(np.float32)
        ms.append(((v * 0.5 + off).astype(np.float32), ip, k))
    oms = [orc.Mesh(v, ip, keys=k, motion_fixed=True) for v, ip, k in ms]
    osc = orc.Scene(oms)
    ids = [ctx.mesh_build(v, ip, keys=k, motion_mode=1) for v, ip, k in ms]
    ctx.scene_build(ids)
    rays = scenes.incoherent_rays(100000, 60, lo=-1.5, hi=1.5)
    rays[:, 7] = scenes.uniform(61, rays.shape[0], 3).astype(np.float32)
    for shadow in (False, True):
        got = ctx.trace_scene(rays, shadow=shadow)
        ref = osc.trace(rays, shadow=shadow)
        ref["geom"] = np.where(ref["geom"] >= 0, np.asarray(ids, np.int32)[np.maximum(ref["geom"], 0)], -1)
        assert_hits_equal(got, ref, keys=("prim", "geom", "t", "u", "v", "w"), what=f"scene shadow={shadow}")


def test_full_size_soup_parity(ctx, orc):
    """The raw-traversal configuration at its stated size: the 1,048,576-
    triangle soup (seed 2) under all 4,194,304 incoherent rays and the
    4,194,304 coherent primaries of a 2048x2048 pinhole, closest hit and any
    hit, every hit compared with the oracle (multithreaded on the host)."""
    v, ip = scenes.triangle_soup(1 << 20, 2)
    geom = ctx.mesh_build(v, ip)
    om = orc.Mesh(v, ip)
    for name, rays in (("incoherent", scenes.incoherent_rays(1 << 22, 2)), ("coherent", scenes.coherent_rays(2048))):
        assert rays.shape[0] == 1 << 22
        for shadow in (False, True):
            assert_hits_equal(ctx.trace_mesh(geom, rays, shadow=shadow), om.trace(rays, shadow=shadow),
                              what=f"1M soup {name} shadow={shadow}")


@pytest.mark.parametrize("tuning", [(0, 0, 0, 0), (1, 0, 0, 0), (3, 0, 0, 0), (5, 0, 0, 0), (8, 0, 0, 4),
                                    (9, 0, 0, 0), (13, 0, 0, 0), (9, 64, 0, 0), (9, 256, 2, 0), (13, 0, 0, 0, 4), (9, 0, 0, 0, 12),
                                    (13, 0, 0, 0, 4, 3), (13, 0, 0, 0, 4, 5), (8, 256, 0, 4, 4, 5),
                                    (29, 0, 0, 0, 4), (17, 0, 0, 0, 0), (25, 256, 0, 0, 8, 3), (21, 64, 0, 0, 2),
                                    (16, 0, 0, 0), (45, 0, 0, 0, 4), (45, 0, 0, 0, 0), (33, 0, 0, 0, 8),
                                    (41, 256, 0, 0, 4, 3), (37, 0, 0, 0, 2)])
def test_every_tuning_is_bit_exact(ctx, orc, tuning):
    """Launch parameters (kernel variant, ray reordering and its key width,
    block size, resident blocks) only change scheduling: hits stay
    bit-exact."""
    v, ip = scenes.triangle_soup(100000, 17, edge=0.006)
    rays = scenes.incoherent_rays(150000, 18)
    geom = ctx.mesh_build(v, ip)
    om = orc.Mesh(v, ip)
    try:
        ctx.set_tuning(*tuning)
        for shadow in (False, True):
            assert_hits_equal(ctx.trace_mesh(geom, rays, shadow=shadow), om.trace(rays, shadow=shadow),
                              what=f"tuning={tuning} shadow={shadow}")
        mv, mip = scenes.motion_soup(20000, 19, edge=0.01)
        mg = ctx.mesh_build(mv, mip, keys=2, motion_mode=1)
        mrays = rays.copy()
        mrays[:, 7] = scenes.uniform(20, mrays.shape[0], 1).astype(np.float32)
        assert_hits_equal(ctx.trace_mesh(mg, mrays), orc.Mesh(mv, mip, keys=2, motion_fixed=True).trace(mrays),
                          what=f"motion tuning={tuning}")
    finally:
        ctx.set_tuning(45, 0, 0, 0, 8)


@pytest.mark.parametrize("tuning", [(13, 0, 0, 0, 4), (45, 0, 0, 0, 8), (45, 0, 0, 0, 0), (1, 0, 0, 0, 0),
                                    (5, 0, 0, 0, 8), (0, 0, 0, 4, 4),
                                    (13, 0, 0, 0, 2, 5), (8, 0, 0, 4, 4), (12, 0, 0, 0, 0, 3)])
def test_two_level_scene_every_tuning(ctx, orc, tuning):
    """The static two-level scene traced by the while-while scene kernel (with
    and without ray reordering, several tail cutoffs) and by the single-loop
    kernel (unsorted, and sorted: tunings 8 and 12 write each hit back
    through the order array): all bit-exact with the oracle, closest and any
    hit."""
    rng = np.random.default_rng(77)
    ms = []
    for i in range(30):
        n = int(rng.integers(1, 8000))
        v, ip = scenes.triangle_soup(n, 700 + i, edge=0.01)
        off = rng.uniform(-1, 1, 3).astype(np.float32)
        ms.append(((v * 0.6 + off).astype(np.float32), ip))
    oms = [orc.Mesh(v, ip) for v, ip in ms]
    osc = orc.Scene(oms)
    ids = [ctx.mesh_build(v, ip) for v, ip in ms]
    ctx.scene_build(ids)
    rays = np.concatenate([scenes.incoherent_rays(70000, 78, lo=-1.5, hi=1.5),
                           scenes.coherent_rays(200, eye=(0.0, 0.0, -3.0), target=(0.0, 0.0, 0.0))])
    try:
        ctx.set_tuning(*tuning)
        for shadow in (False, True):
            got = ctx.trace_scene(rays, shadow=shadow)
            ref = osc.trace(rays, shadow=shadow)
            ref["geom"] = np.where(ref["geom"] >= 0, np.asarray(ids, np.int32)[np.maximum(ref["geom"], 0)], -1)
            assert_hits_equal(got, ref, keys=("prim", "geom", "t", "u", "v", "w"),
                              what=f"scene tuning={tuning} shadow={shadow}")
    finally:
        ctx.set_tuning(45, 0, 0, 0, 8)



@pytest.mark.parametrize("tuning", [(13, 0, 0, 0, 4), (45, 0, 0, 0, 8), (0, 0, 0, 4, 4)])
def test_scene_with_sphere_geoms(ctx, orc, tuning):
    """Analytic sphere geoms among triangle meshes (Sphere.Trace: the nearer
    non-negative root below Tclosest), in both scene kernels."""
    rng = np.random.default_rng(91)
    ms, oms, ids = [], [], []
    for i in range(12):
        v, ip = scenes.triangle_soup(int(rng.integers(100, 3000)), 900 + i, edge=0.01)
        off = rng.uniform(-1, 1, 3).astype(np.float32)
        v = (v * 0.6 + off).astype(np.float32)
        oms.append(orc.Mesh(v, ip))
        ids.append(ctx.mesh_build(v, ip))
    for i in range(8):
        c = rng.uniform(-1, 1, 3).astype(np.float32)
        r = float(rng.uniform(0.05, 0.4))
        oms.append(orc.Sphere(c, r))
        ids.append(ctx.sphere_add(c, r))
    osc = orc.Scene(oms)
    ctx.scene_build(ids)
    rays = np.concatenate([scenes.incoherent_rays(70000, 92, lo=-1.5, hi=1.5),
                           scenes.incoherent_rays(20000, 93, lo=-0.2, hi=0.2)])
    try:
        ctx.set_tuning(*tuning)
        for shadow in (False, True):
            got = ctx.trace_scene(rays, shadow=shadow)
            ref = osc.trace(rays, shadow=shadow)
            ref["geom"] = np.where(ref["geom"] >= 0, np.asarray(ids, np.int32)[np.maximum(ref["geom"], 0)], -1)
            assert_hits_equal(got, ref, keys=("prim", "geom", "t", "u", "v", "w"), what=f"spheres shadow={shadow}")
        assert (got["geom"] >= ids[12]).any()  # some rays end on spheres
    finally:
        ctx.set_tuning(45, 0, 0, 0, 8)


def test_host_trace_equals_device_trace(ctx, orc):
    """A host-pointer trace (rays staged in, hits copied out inside the call)
    of 2,500,001 rays equals the device-pointer trace of the same rays bit
    for bit, and its visit counters equal the oracle's."""
    import torch
    v, ip = scenes.triangle_soup(100000, 41, edge=0.006)
    geom = ctx.mesh_build(v, ip)
    rays = scenes.incoherent_rays(2_500_001, 42)
    dev = torch.from_numpy(np.ascontiguousarray(rays.T)).cuda()
    for shadow in (False, True):
        host = ctx.trace_mesh(geom, rays, shadow=shadow, counters=True)
        d = ctx.trace_mesh(geom, dev, shadow=shadow)
        ctx.sync()  # device-pointer traces are asynchronous on the context's stream
        d = {k: d[k].cpu().numpy() for k in ("prim", "t", "u", "v", "w")}
        assert_hits_equal(host, d, what=f"host vs device shadow={shadow}")
        assert host["stats"]["rays"] == rays.shape[0]
        if not shadow:
            ref = orc.Mesh(v, ip).trace(rays, counters=True)
            c = np.asarray(ref["counters"], np.uint64)
            assert host["stats"]["node_visits"] == int(c[:, 0].sum())
            assert host["stats"]["tri_tests"] == int(c[:, 2].sum())
