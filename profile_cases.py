"""Named workloads for kernel profiling (each runs once and exits 0):

    python profile_cases.py guide        guide inference on 1M vertices
                                                       and one training step of 256K
    python profile_cases.py render_ext   extended path tracer, sphere grid,
                                                       1920x1080, 2 spp, depth 8
    python profile_cases.py render_ext_flat / render_ext_two_level
                                         the same render twice, the scene
                                                       flattened or two-level
    python profile_cases.py render_ref   reference-mode render, small room,
                                                       256x256, 16 iterations
    python profile_cases.py render_ref_f32  the same with float32 shading
    python profile_cases.py jobs         64 uneven jobs in one launch
    python profile_cases.py path_jobs    64 uneven static/motion jobs path traced
                                                       in one call, 256x256, 2 spp, depth 5
    python profile_cases.py build        device QBVH build of the 1M-triangle soup

Inputs are the seeded synthetic scenes of vermeer_gb300.scenes.
"""
from __future__ import annotations

import sys

import numpy as np


def guide(ctx):
    rng = np.random.default_rng(1)
    n = 1 << 20
    pos = rng.random((n, 3)).astype(np.float32)
    nrm = rng.standard_normal((n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.standard_normal((n, 3)).astype(np.float32)
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    lo, hi = np.zeros(3, np.float32), np.ones(3, np.float32)
    ctx.guide_init(1)
    ctx.guide_forward(pos, nrm, wo, lo, hi)
    m = 1 << 18
    ctx.guide_train_step(pos[:m], nrm[:m], wo[:m], wo[:m], np.ones(m, np.float32), lo, hi)


def render_ext(ctx):
    from vermeer_gb300 import scenes
    sc = scenes.sphere_grid()
    ctx.load_scene(sc)
    ctx.render_path(sc["width"], sc["height"], 0, 2, 3, max_depth=8)


def _render_ext_twice(ctx, two_level):
    from vermeer_gb300 import scenes
    sc = scenes.sphere_grid()
    ctx.load_scene(sc)
    for _ in range(2):
        ctx.render_path(sc["width"], sc["height"], 0, 2, 3, max_depth=8, two_level=two_level)


def render_ext_flat(ctx):
    _render_ext_twice(ctx, False)


def render_ext_two_level(ctx):
    _render_ext_twice(ctx, True)


def render_ref(ctx):
    from vermeer_gb300 import scenes
    sc = scenes.small_room(16384, seed=1)
    ctx.load_scene(sc)
    ctx.render(256, 256, 0, 16, 7)


def render_ref_f32(ctx):
    from vermeer_gb300 import scenes
    sc = scenes.small_room(16384, seed=1)
    ctx.load_scene(sc)
    ctx.render(256, 256, 0, 16, 7, f32=True)


def jobs(ctx):
    import torch
    from vermeer_gb300 import scenes
    sizes = np.exp(np.log(1000) + (np.log(200000) - np.log(1000)) * scenes.uniform(4, 64, 0)).astype(int)
    cam = scenes.coherent_rays(256)
    js = []
    for j, nt in enumerate(sizes):
        motion = j % 2 == 1
        v, ip = scenes.motion_soup(int(nt), 400 + j) if motion else scenes.triangle_soup(int(nt), 400 + j)
        g = ctx.mesh_build(v, ip, keys=2 if motion else 1, motion_mode=1)
        rays = cam.copy()
        if motion:
            rays[:, 7] = scenes.uniform(500 + j, rays.shape[0], 7).astype(np.float32)
        js.append((g, torch.from_numpy(np.ascontiguousarray(rays.T)).cuda()))
    ctx.trace_jobs(js)


def path_jobs(ctx):
    from vermeer_gb300 import scenes
    bj = scenes.batched_jobs()
    ids = [ctx.mesh_build(m["verts"], m["idxp"], keys=m.get("keys", 1), motion_mode=m.get("motion_mode", 0))
           for m in bj["meshes"]]
    ctx.set_shaders(bj["shaders"])
    for g in ids:
        ctx.mesh_set_shading(g, [0])
    ctx.set_lights([])
    ctx.set_quad_lights([])
    ctx.set_env_light(bj["env"])
    jobs = [dict(geom=g, width=bj["width"], height=bj["height"], camera=c) for g, c in zip(ids, bj["cameras"])]
    ctx.render_path_jobs(jobs, 0, 2, 5, max_depth=5)


def build(ctx):
    from vermeer_gb300 import scenes
    from vermeer_gb300.api import BUILD_DEVICE
    v, ip = scenes.triangle_soup(1 << 20, 2)
    ctx.set_builder(BUILD_DEVICE)
    ctx.mesh_build(v, ip)


CASES = {"guide": guide, "render_ext": render_ext, "render_ext_flat": render_ext_flat,
         "render_ext_two_level": render_ext_two_level, "render_ref": render_ref, "render_ref_f32": render_ref_f32,
         "jobs": jobs, "path_jobs": path_jobs, "build": build}


def main(argv):
    if len(argv) != 1 or argv[0] not in CASES:
        print(__doc__)
        return 2
    import vermeer_gb300 as vg
    ctx = vg.Context(0)
    CASES[argv[0]](ctx)
    ctx.sync()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
