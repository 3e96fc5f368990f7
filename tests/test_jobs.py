"""Batched uneven jobs (vmr_trace_jobs) and the per-mesh autotuner
(vmr_autotune).  Neither has a reference counterpart (the reference traces
one scene per process with fixed settings); both must leave every hit
bit-identical to the single-mesh trace, which the oracle pins."""
import numpy as np
import pytest

from conftest import assert_hits_equal
from vermeer_gb300 import scenes


def _jobs_workload(n_jobs=10, seed=4):
    """Meshes of log-uniform size in [1k, 60k] triangles, every other one with
    two-key linear motion (velocity in a 0.05 ball), and uneven ray counts
    (camera-like rays through the soup, times uniform in [0, 1))."""
    sizes = np.exp(np.log(1000) + (np.log(60000) - np.log(1000)) * scenes.uniform(seed, n_jobs, 0)).astype(int)
    out = []
    for j, nt in enumerate(sizes):
        motion = j % 2 == 1
        if motion:
            v, ip = scenes.motion_soup(int(nt), seed * 100 + j, velocity=0.05, edge=0.01)
        else:
            v, ip = scenes.triangle_soup(int(nt), seed * 100 + j, edge=0.01)
        nr = int(2000 + 30000 * scenes.uniform(seed, n_jobs, 1)[j])
        rays = scenes.incoherent_rays(nr, seed * 1000 + j)
        rays[:, 7] = scenes.uniform(seed * 1000 + j, nr, 7).astype(np.float32)
        out.append((v, ip, motion, rays))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("shadow", [False, True])
def test_jobs_match_single_traces(ctx, orc, shadow):
    import torch
    work = _jobs_workload()
    jobs, ref = [], []
    for v, ip, motion, rays in work:
        g = ctx.mesh_build(v, ip, keys=2 if motion else 1, motion_mode=1)
        d = torch.from_numpy(np.ascontiguousarray(rays.T)).cuda()
        jobs.append((g, d))
        ref.append(ctx.trace_mesh(g, d, shadow=shadow))
    jobs.append((jobs[0][0], torch.zeros((8, 0), dtype=torch.float32, device="cuda")))  # an empty job
    outs, st = ctx.trace_jobs(jobs, shadow=shadow)
    assert st["rays"] == sum(r.shape[0] for *_, r in work)
    for j, (out, r) in enumerate(zip(outs, ref)):
        got = {k: out[k].cpu().numpy() for k in ("prim", "t", "u", "v", "w")}
        exp = {k: r[k].cpu().numpy() for k in ("prim", "t", "u", "v", "w")}
        keys = ("prim",) if shadow else ("prim", "t", "u", "v", "w")
        if shadow:  # any hit: whether a ray hits is fixed; which prim need not be
            assert np.array_equal(got["prim"] >= 0, exp["prim"] >= 0), j
        else:
            assert_hits_equal(got, exp, keys=keys, what=f"job {j}")
    # one static and one motion job against the oracle
    for j in (0, 1):
        v, ip, motion, rays = work[j]
        om = orc.Mesh(v, ip, keys=2 if motion else 1, motion_fixed=motion)
        o = om.trace(rays, shadow=shadow)
        got = {k: outs[j][k].cpu().numpy() for k in ("prim", "t", "u", "v", "w")}
        if shadow:
            assert np.array_equal(got["prim"] >= 0, o["prim"] >= 0)
        else:
            assert_hits_equal(got, o, what=f"job {j} vs oracle")


@pytest.mark.gpu
def test_autotune_picks_a_config_and_stays_exact(ctx, orc):
    v, ip = scenes.triangle_soup(200000, 31, edge=0.005)
    rays = scenes.incoherent_rays(300000, 32)
    g = ctx.mesh_build(v, ip)
    best, ms, tried = ctx.autotune(g, rays)
    assert tried >= 20 and ms > 0
    assert best["kernel"] in (0, 1, 5, 8, 9, 13, 29, 41, 45) and best["sort_bits"] in (0, 3, 4, 5)
    try:
        assert_hits_equal(ctx.trace_mesh(g, rays), orc.Mesh(v, ip).trace(rays), what="after autotune")
    finally:
        ctx.clear_tuning(g)
