"""Reference-mode render path: core.Render (core/render.go:66-218) with
ShaderStd, TriLight and the hero-wavelength spectrum.

CPU tests pin properties of the oracle renderer; GPU tests compare
vmr_render with the oracle image at equal samples per pixel.

Tolerance.  Both sides run the same float32 operation sequence without
contraction; transcendentals are float64 on both sides, rounded to float32.
CUDA's float64 sin/cos/tan/atan/acos are within 2 ulp of the exact value,
so the float32 result can differ from the host's by one float32 ulp in
the rare case that the exact value lies within 2^-29 relative of a float32
rounding boundary.  A pixel is "equal" when all three channels agree within
|a-b| <= 1e-5 * (1 + |b|); the test requires 99.9% equal pixels and a mean
absolute difference below 1e-6 over the image.
"""
import numpy as np
import pytest

from vermeer_gb300 import scenes

W = H = 64
ITERS = 4
SEED = 7
REL = 1e-5
FRAC_EQUAL = 0.999
MEAN_ABS = 1e-6


@pytest.fixture(scope="module")
def room():
    return scenes.small_room(4096, seed=3)


@pytest.fixture(scope="module")
def oracle_render(orc, room):
    return orc.Render(room)


def _compare(got, ref):
    assert got.shape == ref.shape
    assert not np.isnan(got).any() and not np.isnan(ref).any()
    ok = np.abs(got - ref) <= REL * (1.0 + np.abs(ref))
    frac = ok.all(-1).mean()
    mean_abs = np.abs(got - ref).mean()
    return frac, mean_abs


# ------------------------------------------------------------------ CPU ----
def test_oracle_render_deterministic(oracle_render):
    a = oracle_render.run(W, H, 0, 2, SEED, nthreads=1)
    b = oracle_render.run(W, H, 0, 2, SEED, nthreads=4)
    assert a.tobytes() == b.tobytes()


def test_oracle_render_iterations_fold(oracle_render):
    """Iterations [0,4) in one call equal [0,2) then [2,4): the running mean
    buf = (buf*j + c)/(j+1) is folded per iteration (core/render.go:127-129)."""
    full = oracle_render.run(W, H, 0, 4, SEED)
    part = oracle_render.run(W, H, 0, 2, SEED)
    part = oracle_render.run(W, H, 2, 2, SEED, fb=part)
    assert full.tobytes() == part.tobytes()


def test_oracle_render_image_sane(oracle_render):
    fb = oracle_render.run(W, H, 0, ITERS, SEED)
    assert np.isfinite(fb).all()
    assert (fb >= 0).all()
    lit = fb.sum(-1) > 0
    assert 0.5 < lit.mean() < 1.0
    # the emitters are visible through the ceiling opening: radiance 10 x
    # the white spectrum, folded with weight (j+1)/(j+2) etc.
    assert fb.max() > 5.0


def test_oracle_render_seed_changes_image(oracle_render):
    a = oracle_render.run(W, H, 0, 1, SEED)
    b = oracle_render.run(W, H, 0, 1, SEED + 1)
    assert a.tobytes() != b.tobytes()


def test_render_scene_has_no_degenerate_light_planes(room):
    """No surface of the room crosses a light's plane (a shading point in
    the plane makes the reference's spherical-triangle sampling NaN)."""
    ys = {float(l["p0"][1]) for l in room["lights"]}
    assert len(ys) == len(room["lights"])
    for m in room["meshes"][:2]:
        assert m["verts"][:, 1].max() < min(ys)


# ------------------------------------------------------------------ GPU ----
@pytest.mark.gpu
def test_render_matches_oracle(ctx, room, oracle_render):
    ctx.load_scene(room)
    ref = oracle_render.run(W, H, 0, ITERS, SEED)
    got, st = ctx.render(W, H, 0, ITERS, SEED)
    frac, mean_abs = _compare(got, ref)
    assert frac >= FRAC_EQUAL, (frac, mean_abs)
    assert mean_abs <= MEAN_ABS, (frac, mean_abs)
    assert st["samples"] == W * H * ITERS
    assert st["camera_rays"] == W * H * ITERS
    assert st["shadow_rays"] > 0


@pytest.mark.gpu
def test_render_batches_are_exact(ctx, room):
    """Splitting the iterations over batches (max_batch_samples) or over
    calls does not change a bit."""
    ctx.load_scene(room)
    one, _ = ctx.render(W, H, 0, ITERS, SEED)
    small, _ = ctx.render(W, H, 0, ITERS, SEED, max_batch_samples=W * H)
    assert one.tobytes() == small.tobytes()
    part, _ = ctx.render(W, H, 0, 1, SEED)
    part, _ = ctx.render(W, H, 1, ITERS - 1, SEED, fb=part)
    assert one.tobytes() == part.tobytes()


@pytest.mark.gpu
def test_render_non_square_matches_oracle(ctx, orc):
    sc = scenes.small_room(2048, seed=5, light_samples=2)
    ctx.load_scene(sc)
    r = orc.Render(sc)
    ref = r.run(48, 32, 3, 2, 11)
    got, _ = ctx.render(48, 32, 3, 2, 11)
    frac, mean_abs = _compare(got, ref)
    assert frac >= FRAC_EQUAL and mean_abs <= MEAN_ABS, (frac, mean_abs)


# ----------------------------------------------- DiskLight and thin lens ----
def test_oracle_disk_light_room_sane(orc):
    sc = scenes.small_room_disk(2048, seed=4)
    fb = orc.Render(sc).run(32, 32, 0, 8, 5)
    assert np.isfinite(fb).all() and (fb >= 0).all()
    assert 0.3 < (fb.sum(-1) > 0).mean() <= 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [0, 1, 2])
def test_render_disk_light_thin_lens_matches_oracle(ctx, orc, samples):
    """DiskLight area sampling and ValidSample (one light sample without MIS
    at samples=0, MIS with 1+1 and 2+2) through a thin-lens camera."""
    sc = scenes.small_room_disk(2048, seed=4, light_samples=samples)
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(40, 40, 0, 3, 9)
    got, _ = ctx.render(40, 40, 0, 3, 9)
    frac, mean_abs = _compare(got, ref)
    assert frac >= FRAC_EQUAL and mean_abs <= MEAN_ABS, (frac, mean_abs)


# ------------------------------------------------------ mirror recursion ----
def test_oracle_mirror_room_sane(orc):
    sc = scenes.small_room_mirror(2048, seed=6)
    fb = orc.Render(sc).run(32, 32, 0, 4, 5)
    assert np.isfinite(fb).all() and (fb >= 0).all() and fb.mean() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [0, 1])
def test_render_mirror_recursion_matches_oracle(ctx, orc, samples):
    """Mirror reflections (core.Trace recursion, one light sample per light
    below the camera level) down to level 3."""
    sc = scenes.small_room_mirror(2048, seed=6, light_samples=samples)
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(48, 48, 0, 3, 13)
    got, st = ctx.render(48, 48, 0, 3, 13)
    frac, mean_abs = _compare(got, ref)
    assert frac >= FRAC_EQUAL and mean_abs <= MEAN_ABS, (frac, mean_abs)
    assert st["camera_rays"] == 48 * 48 * 3


# ------------------------------------------- sphere geoms and SphereLight ----
def test_oracle_sphere_room_sane(orc):
    sc = scenes.small_room_spheres(2048, seed=8)
    fb = orc.Render(sc).run(32, 32, 0, 4, 5)
    assert np.isfinite(fb).all() and (fb >= 0).all() and fb.mean() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("samples", [0, 1])
def test_render_spheres_match_oracle(ctx, orc, samples):
    """Analytic sphere geoms (Lambert, GGX, mirror) and a SphereLight (cone
    sampling, ValidSample) next to the TriLights."""
    sc = scenes.small_room_spheres(2048, seed=8, light_samples=samples)
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(48, 48, 0, 3, 17)
    got, _ = ctx.render(48, 48, 0, 3, 17)
    frac, mean_abs = _compare(got, ref)
    assert frac >= FRAC_EQUAL and mean_abs <= MEAN_ABS, (frac, mean_abs)


# ---------------------------------------------------------- motion blur ----
def test_oracle_motion_room_sane(orc):
    sc = scenes.small_room_motion(2048, seed=9)
    fb = orc.Render(sc).run(32, 32, 0, 4, 5)
    assert np.isfinite(fb).all() and (fb >= 0).all() and fb.mean() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1])
def test_render_motion_blur_matches_oracle(ctx, orc, mode):
    """A two-key motion soup rendered over the shutter (each sample's VdC
    time): the motion traversal and the lerped hit attributes of
    TraceMotionElems, in both leaf-indexing modes."""
    sc = scenes.small_room_motion(2048, seed=9, motion_mode=mode)
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(48, 48, 0, 3, 19)
    got, _ = ctx.render(48, 48, 0, 3, 19)
    frac, mean_abs = _compare(got, ref)
    assert frac >= FRAC_EQUAL and mean_abs <= MEAN_ABS, (frac, mean_abs)
