"""Pins of the CPU oracle: against the reference's own data (the QMC tables),
hand-derived known answers, mathematical properties, an independent
brute-force intersector, and the committed golden traversal fixture."""
import os

import numpy as np
import pytest

from conftest import assert_hits_equal

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


# ------------------------------------------------------------------ QMC ---
def test_tables_equal_reference(orc):
    """Tables derived from the generator matrices equal the reference's
    vdcSobolMatrices / vdcSobolMatricesInv (math/ldseq/vdc_sobol_matrices52.go)
    for every m the reference lists."""
    g = np.load(os.path.join(GOLDEN, "vdc_sobol_tables.npz"))
    for m in range(1, 27):
        f, v = orc.vdc_sobol_tables(m)
        if m <= 25:
            assert np.array_equal(f, g["fwd"][m]), f"fwd m={m}"
        assert np.array_equal(v, g["inv"][m]), f"inv m={m}"


def _vdc_py(i, s):  # ldseq.go:55-75 by string reversal
    b = int(format(i & (2**64 - 1), "064b")[::-1], 2)
    return ((s ^ b) & (2**64 - 1)) >> 12


def _sobol_py(i, s):  # ldseq.go:83-96, columns from Pascal's triangle mod 2
    r = s >> 12
    k = 0
    while i:
        if i & 1:
            col = 0
            for j in range(k + 1):  # C(k, j) odd  <=>  j & k == j
                if j & k == j and j < 52:
                    col |= 1 << (51 - j)
            r ^= col
        i >>= 1
        k += 1
    return r


def test_vdc_sobol_known_answers(orc):
    rng = np.random.default_rng(1)
    cases = [(0, 0), (1, 0), (2, 0), (3, 0), (0x12345, 0), (2**40 + 7, 0)]
    cases += [(int(a), int(b)) for a, b in zip(rng.integers(0, 2**62, 200), rng.integers(0, 2**63, 200))]
    for i, s in cases:
        assert orc.vdc(i, s) == _vdc_py(i, s), (i, s)
        assert orc.sobol(i, s) == _sobol_py(i, s), (i, s)
    # hand values: index 1 -> 0.5 in both dimensions; index 2 -> 0.25 / 0.75
    assert orc.vdc(1, 0) == 1 << 51 and orc.sobol(1, 0) == 1 << 51
    assert orc.vdc(2, 0) == 1 << 50 and orc.sobol(2, 0) == 3 << 50


def test_sobol_02_net(orc):
    """The first 2^k points of (VdC, Sobol) form a (0,k,2)-net: every
    elementary interval of area 2^-k holds exactly one point."""
    k = 8
    pts = [(orc.vdc(i, 0), orc.sobol(i, 0)) for i in range(1 << k)]
    for a in range(k + 1):
        b = k - a
        cells = {(x >> (52 - a), y >> (52 - b)) for x, y in pts}
        assert len(cells) == 1 << k, (a, b)


def test_vdc_sobol_histogram_is_flat(orc):
    """The histogram check of the reference's QMC test (core/qmc_test.go:
    10-35 bins (RadicalInvVdC(k), RadicalInvSobol(k)) on a grid and writes
    the counts out): for a power-of-two point count the (0,2)-sequence
    makes every cell hold the same number of points; here 2^18 points on a
    256 x 256 grid, 4 per cell."""
    n, res = 1 << 18, 256
    x = np.array([orc.vdc(i, 0) for i in range(n)], np.uint64) >> np.uint64(52 - 8)
    y = np.array([orc.sobol(i, 0) for i in range(n)], np.uint64) >> np.uint64(52 - 8)
    counts = np.bincount((x + y * np.uint64(res)).astype(np.int64), minlength=res * res)
    assert counts.min() == counts.max() == 4


@pytest.mark.parametrize("m", [3, 5, 12])
def test_raster_xy_lands_in_pixel(orc, m):
    """RasterXY(m, frame, px, py) returns the frame-th sample of pixel
    (px,py): the sample lies in [px,px+1) x [py,py+1) and frames give
    distinct sample indices (raster.go:50-57)."""
    rng = np.random.default_rng(m)
    res = 1 << m
    for _ in range(40):
        px, py = int(rng.integers(0, res)), int(rng.integers(0, res))
        seen = set()
        for frame in range(16):
            idx, rx, ry = orc.raster_xy(m, frame, px, py)
            assert px <= rx < px + 1 and py <= ry < py + 1, (px, py, frame, rx, ry)
            assert (orc.vdc(idx, 0) >> (52 - m)) == px and (orc.sobol(idx, 0) >> (52 - m)) == py
            seen.add(idx)
        assert len(seen) == 16


# ------------------------------------------------------------ traversal ---
def test_leaf_encoding_roundtrip(orc):
    """SetLeaf / LeafBase / LeafCount (qbvh/qbvh.go:61-93) as stored by the
    oracle's builder: every leaf decodes to a disjoint range covering all
    triangles exactly once."""
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(5000, 3)
    ex = orc.Mesh(v, ip).export()
    covered = np.zeros(5000, np.int32)
    for nd in ex["nodes"]:
        for c in nd["children"]:
            if c < -1:
                c = int(np.uint32(np.int32(c)))
                base, count = (c & 0x7ffffff) >> 4, (c & 0xF) + 1
                covered[base:base + count] += 1
    assert np.all(covered == 1)
    assert sorted(ex["accel_idx"].tolist()) == list(range(5000))


def _brute_force_t(verts, rays):
    """Closest t over all triangles with the reference's watertight test in
    float32 numpy arithmetic (numpy never fuses), written independently of
    the oracle's traversal.  Returns +inf for misses."""
    tri = verts.reshape(-1, 3, 3).astype(np.float32)
    out = np.full(rays.shape[0], np.inf, np.float32)
    eps = np.float32(1.19209290e-07)
    for r, ray in enumerate(rays):
        P = ray[0:3].astype(np.float32)
        D = ray[3:6].astype(np.float32)
        a = np.abs(D)
        kz = 0
        if a[1] > a[2]:
            if a[1] > a[0]:
                kz = 1
        elif a[2] > a[0]:
            kz = 2
        kx = (kz + 1) % 3
        ky = (kx + 1) % 3
        if D[kz] < 0:
            kx, ky = ky, kx
        z = np.float64(D[kz])
        S = np.array([np.float64(D[kx]) / z, np.float64(D[ky]) / z, 1.0 / z], np.float32)
        A = tri[:, 0, :] - P
        B = tri[:, 1, :] - P
        C = tri[:, 2, :] - P
        Ax = A[:, kx] - S[0] * A[:, kz]
        Ay = A[:, ky] - S[1] * A[:, kz]
        Bx = B[:, kx] - S[0] * B[:, kz]
        By = B[:, ky] - S[1] * B[:, kz]
        Cx = C[:, kx] - S[0] * C[:, kz]
        Cy = C[:, ky] - S[1] * C[:, kz]
        U = Cx * By - Cy * Bx
        V = Ax * Cy - Ay * Cx
        W = Bx * Ay - By * Ax
        z0 = (U == 0) | (V == 0) | (W == 0)
        if z0.any():
            U[z0] = (Cx[z0].astype(np.float64) * By[z0] - Cy[z0].astype(np.float64) * Bx[z0]).astype(np.float32)
            V[z0] = (Ax[z0].astype(np.float64) * Cy[z0] - Ay[z0].astype(np.float64) * Cx[z0]).astype(np.float32)
            W[z0] = (Bx[z0].astype(np.float64) * Ay[z0] - By[z0].astype(np.float64) * Ax[z0]).astype(np.float32)
        ok = ~(((U < 0) | (V < 0) | (W < 0)) & ((U > 0) | (V > 0) | (W > 0)))
        det = (U + V) + W
        ok &= det != 0
        T = S[2] * ((U * A[:, kz] + V * B[:, kz]) + W * C[:, kz])
        sgn = np.where(det < 0, np.float32(-1), np.float32(1))
        ok &= ~((T * sgn) < eps * (det * sgn))
        t = np.where(ok, T * (np.float32(1) / np.where(det == 0, np.float32(1), det)), np.float32(np.inf))
        t = np.where(t <= ray[6], t, np.float32(np.inf))
        out[r] = t.min()
    return out


def test_oracle_matches_brute_force(orc):
    """The ordered QBVH traversal finds the same closest t as testing every
    triangle (no hit is missed, no farther hit is kept)."""
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(3000, 21, edge=0.03)
    rays = scenes.incoherent_rays(400, 22)
    res = orc.Mesh(v, ip).trace(rays)
    bf = _brute_force_t(v, rays)
    hit = res["prim"] >= 0
    assert np.array_equal(np.isfinite(bf), hit)
    assert np.array_equal(res["t"][hit], bf[hit])


def test_golden_traversal_fixture(orc):
    """The oracle reproduces the committed closest-hit and any-hit answers
    bit for bit on this machine."""
    g = np.load(os.path.join(GOLDEN, "traversal_small.npz"))
    for case in ("soup64", "soup2k", "soup8k"):
        m = orc.Mesh(g[f"{case}__verts"], g[f"{case}__idxp"])
        rays = g[f"{case}__rays"]
        for mode, shadow in (("ch", False), ("any", True)):
            got = m.trace(rays, shadow=shadow)
            ref = {k: g[f"{case}__{mode}_{k}"] for k in ("prim", "t", "u", "v", "w")}
            assert_hits_equal(got, ref, what=f"{case}/{mode}")


def test_any_hit_agrees_with_closest_on_hit_or_miss(orc):
    from vermeer_gb300 import scenes
    v, ip = scenes.triangle_soup(20000, 31)
    m = orc.Mesh(v, ip)
    rays = scenes.incoherent_rays(5000, 32)
    a = m.trace(rays)
    b = m.trace(rays, shadow=True)
    assert np.array_equal(a["prim"] >= 0, b["prim"] >= 0)
    assert np.all(b["t"][b["prim"] >= 0] >= a["t"][b["prim"] >= 0])


def test_motion_faithful_vs_fixed_differ_only_by_face_mapping(orc):
    """At time 0.5 boxes and vertices are lerped; the fixed mode reports the
    original face ids.  With an identity build permutation both modes agree,
    which holds for a single-leaf mesh."""
    from vermeer_gb300 import scenes
    v, ip = scenes.motion_soup(12, 41, velocity=0.05, edge=0.2)
    rays = scenes.incoherent_rays(500, 42)
    rays[:, 7] = 0.5
    fa = orc.Mesh(v, ip, keys=2, motion_fixed=False).trace(rays)
    fx = orc.Mesh(v, ip, keys=2, motion_fixed=True).trace(rays)
    ex = orc.Mesh(v, ip, keys=2, motion_fixed=True).export()
    if np.array_equal(ex["accel_idx"], np.arange(12)):
        assert_hits_equal(fa, fx, what="motion 1-leaf")
    assert (fx["prim"] >= 0).any()
