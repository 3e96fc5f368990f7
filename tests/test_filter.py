"""Pixel filters for filter importance sampling (builtin/filter): the
GaussianFilter and AiryFilter tables (CreateSampler, filter.go:87-166) and
Sampler.WarpSample (filter.go:40-80), applied to the RasterXY sample inside
its pixel before the camera ray is made (core/render.go:99-107).

CPU tests pin the oracle's restatement by properties the reference's code
implies (hand-derived), and check libvmr's host warp (vmr_pixel_filter_warp,
the function the camera kernels run) against the oracle bit for bit.  GPU
tests compare filtered renders with the oracle: reference mode to the usual
render tolerance, the extended mode sample for sample.

Tolerance: the warps are float64 integer-free arithmetic in the same
operation order on both sides, and the tables are built on the host by
both, so warps must be bit-identical.
"""
import numpy as np
import pytest

import vermeer_gb300 as vg
from vermeer_gb300 import scenes

GAUSS = {"kind": 1}
AIRY = {"kind": 2}
AIRY_EVEN = {"kind": 2, "res": 48}
GAUSS_WIDE = {"kind": 1, "res": 33, "width": 3.0}


def _samples(n=20000, seed=1):
    rng = np.random.default_rng(seed)
    r0, r1 = rng.random(n), rng.random(n)
    # edges: exact zeros, the largest double below 1, the first-cell branch
    r0[:4] = [0.0, np.nextafter(1.0, 0.0), 1e-9, 0.5]
    r1[:4] = [np.nextafter(1.0, 0.0), 0.0, 0.5, 1e-9]
    return r0, r1


def test_oracle_gaussian_tables(orc):
    cdfV, cdfVU = orc.filter_tables(GAUSS)
    assert cdfV.shape == (17,) and cdfVU.shape == (17, 17)
    assert np.all(np.diff(cdfV) >= 0) and abs(cdfV[-1] - 1.0) < 1e-12
    assert np.all(np.diff(cdfVU, axis=1) >= 0) and np.allclose(cdfVU[:, -1], 1.0)
    # the filter is symmetric in u: the marginal CDF is symmetric about 1/2
    pV = np.diff(np.concatenate([[0.0], cdfV]))
    assert np.allclose(pV, pV[::-1], rtol=1e-12, atol=1e-15)


def test_oracle_gaussian_warp_known_answers(orc):
    """Hand-derived from WarpSample: r0 = r1 = 1/2 falls in the middle cell
    i = 8 with du = 1/2 (symmetric table), so u = v = -1 + 2*(8.5)/16 = 1/16.
    r0 = 0 takes the first-cell branch, u = -1 + (0/cdfV[0])/2 = -1; the
    column u = -1 is zero except at v = 0 (the cutoff is q > 1), so its CDF
    row is 0 up to index 7 and 1 from index 8: r1 = 0 or 0.3 lands in cell 8
    with dv = r1, v = -1 + 2*(8 + r1)/16."""
    u, v = orc.filter_warp(GAUSS, np.array([0.5, 0.0, 0.0]), np.array([0.5, 0.0, 0.3]))
    assert np.allclose(u, [0.0625, -1.0, -1.0], rtol=0, atol=1e-12), u
    assert np.allclose(v, [0.0625, 0.0, 0.0375], rtol=0, atol=1e-12), v
    cdfV, cdfVU = orc.filter_tables(GAUSS)
    assert np.array_equal(cdfVU[0], np.r_[np.zeros(8), np.ones(9)])


def test_oracle_airy_default_is_nan_and_warps_nothing(orc):
    """At res 49 the grid has the point q = 0, where 2 J1(v)/v is 0/0: the
    normalisation turns every table entry into NaN, every comparison
    fails and WarpSample returns (0, 0) (the reference's behaviour)."""
    cdfV, _ = orc.filter_tables(AIRY)
    assert np.isnan(cdfV).all()
    r0, r1 = _samples(1000)
    u, v = orc.filter_warp(AIRY, r0, r1)
    assert not u.any() and not v.any()
    cdfV, _ = orc.filter_tables(AIRY_EVEN)
    assert np.isfinite(cdfV).all() and abs(cdfV[-1] - 1.0) < 1e-12


@pytest.mark.parametrize("f", [GAUSS, AIRY, AIRY_EVEN, GAUSS_WIDE], ids=["gauss", "airy", "airy48", "gauss33"])
def test_lib_warp_matches_oracle(orc, f):
    r0, r1 = _samples()
    ru, rv = orc.filter_warp(f, r0, r1)
    gu, gv = vg.pixel_filter_warp(f["kind"], r0, r1, res=f.get("res", 0), width=f.get("width", 0.0),
                                  peak=f.get("peak", 0.0))
    assert np.array_equal(gu.view(np.uint64), ru.view(np.uint64))
    assert np.array_equal(gv.view(np.uint64), rv.view(np.uint64))


def test_lib_warp_rejects_bad_filters():
    with pytest.raises(vg.VmrError):
        vg.pixel_filter_warp(7, [0.5], [0.5])
    with pytest.raises(vg.VmrError):
        vg.pixel_filter_warp(vg.FILTER_GAUSSIAN, [0.5], [0.5], res=1)
    u, v = vg.pixel_filter_warp(vg.FILTER_BOX, [0.3], [0.7])
    assert u[0] == 0.0 and v[0] == 0.0


# ------------------------------------------------------------------ GPU ----
REL = 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("f", [GAUSS, AIRY_EVEN], ids=["gauss", "airy48"])
def test_render_with_filter_matches_oracle(ctx, orc, f):
    sc = dict(scenes.small_room(2048, seed=6), pixel_filter=f)
    ctx.load_scene(sc)
    ref = orc.Render(sc).run(48, 40, 0, 3, 9)
    got, _ = ctx.render(48, 40, 0, 3, 9)
    ok = (np.abs(got - ref) <= REL * (1.0 + np.abs(ref))).all(-1).mean()
    assert ok >= 0.999 and np.abs(got - ref).mean() <= 1e-6, ok
    # the filter changes the image
    ctx.set_pixel_filter(vg.FILTER_BOX)
    box, _ = ctx.render(48, 40, 0, 3, 9)
    assert not np.array_equal(box, got)


@pytest.mark.gpu
def test_path_render_with_filter_matches_float_oracle(ctx, orc):
    sc = dict(scenes.small_room_ext(1024, seed=8), pixel_filter=GAUSS)
    ctx.load_scene(sc)
    got, _ = ctx.render_path(32, 32, 0, 4, 5, max_depth=4)
    ref, _ = orc.Render(sc).run_path(32, 32, 0, 4, 5, max_depth=4, precision=32)
    ok = (np.abs(got - ref) <= REL * (1.0 + np.abs(ref))).all(-1).mean()
    assert ok >= 0.995, ok


# ------------------------------------------------------- output drivers ----
def _rgbe_inputs():
    rng = np.random.default_rng(3)
    fb = (rng.random((37, 53, 3)) * 4.0).astype(np.float32) ** 3
    fb[0, :5] = [[0, 0, 0], [1e-7, 5e-7, 9e-7], [1e-6, 0, 0], [np.inf, 1, 2], [np.nan, 0.5, 0.25]]
    fb[1, :4] = [[1e30, 3e29, 1e-30], [0.5, 0.5, 0.5], [1.0, 2.0, 4.0], [-1.5, 3.0, 0.0]]
    fb[2, :3] = [[3.4e38, 1.0, 0.0], [255.0, 256.0, 257.0], [0.999, 0.0, 0.0]]
    return fb


def test_oracle_rgbe_known_answers(orc):
    """Hand-derived from convertRGBToRGBE: 0.5 = 0.5 * 2^0 -> m = 0.5, e = 0,
    df = 0.5*255.999/0.5 = 255.999, byte(127.9995) = 127, exponent byte 128;
    (1, 2, 4): d = 4 = 0.5 * 2^3, df = 31.999875 -> 31, 63, 127, 131;
    anything below 1e-6 is four zero bytes; the bottom image row comes
    first."""
    fb = np.zeros((2, 3, 3), np.float32)
    fb[1, 0] = [0.5, 0.5, 0.5]
    fb[1, 1] = [1.0, 2.0, 4.0]
    fb[0, 2] = [5e-7, 0, 0]
    out = orc.encode_rgbe(fb)
    assert out[0, 0].tolist() == [127, 127, 127, 128]
    assert out[0, 1].tolist() == [31, 63, 127, 131]
    assert out[1, 2].tolist() == [0, 0, 0, 0]


@pytest.mark.gpu
def test_encode_rgbe_matches_oracle(ctx, orc, tmp_path):
    import torch
    fb = _rgbe_inputs()
    ref = orc.encode_rgbe(fb)
    assert np.array_equal(ctx.encode_rgbe(fb), ref)
    dev = ctx.encode_rgbe(torch.from_numpy(fb).cuda())
    assert np.array_equal(dev.cpu().numpy(), ref)
    # a rendered frame through the OutputHDR path
    sc = scenes.small_room(1024, seed=2)
    ctx.load_scene(sc)
    img, _ = ctx.render(64, 48, 0, 2, 3)
    p = tmp_path / "out.hdr"
    ctx.write_hdr(str(p), img)
    data = p.read_bytes()
    head = b"#?RADIANCE\n# vermeer_gb300\nFORMAT=32-bit_rle_rgbe\n\n+Y 48 +X 64\n"
    assert data.startswith(head) and data[len(head):] == orc.encode_rgbe(img).tobytes()
