"""The path-guiding network (no reference counterpart): the CPU oracle
(oracle/orc_mlp.cpp) against finite differences and an independent torch
autograd model, and the tensor-core kernels (vermeer_gb300/csrc/guide.cu)
against the oracle's bf16 mode.

Tolerances.  The kernels round weights, layer inputs and deltas to bf16 and
accumulate in float32 in the tensor core's order; the oracle's precision-16
mode makes the same roundings and accumulates in its own order, and computes
the input encoding in float64 (the kernel uses float32 sincospi), so a
rounding can land on the other side of a bf16 tie.  Outputs: relative RMS
difference <= 1e-2 over the batch.  Weight gradients (sums over the batch):
relative L2 difference <= 3e-2 and cosine >= 0.999.
"""
import numpy as np
import pytest

NW = 20032
AMAX = 0.9


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 3)).astype(np.float32) * 2 - 1
    nrm = rng.standard_normal((n, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.standard_normal((n, 3)).astype(np.float32)
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    om = rng.standard_normal((n, 3)).astype(np.float32)
    om /= np.linalg.norm(om, axis=1, keepdims=True)
    wt = (rng.random(n) + 0.25).astype(np.float32)
    return pos, nrm, wo, om, wt


def _weights(seed, scale=0.12):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(NW) * scale).astype(np.float32)


LO = np.array([-1, -1, -1], np.float32)
HI = np.array([1, 1, 1], np.float32)


# ------------------------------------------------------------------ CPU ----
def test_oracle_layout(orc):
    assert orc.Guide.n_weights() == NW == 64 * 80 + 3 * 64 * 64 + 41 * 64


def _bsdf_pdf(nrm, om):
    """Cosine-hemisphere density of om about nrm (0 below the surface)."""
    return np.maximum((nrm * om).sum(1), 0.0).astype(np.float32) / np.float32(np.pi)


@pytest.mark.parametrize("mixed", [False, True])
def test_oracle_gradient_matches_finite_differences(orc, mixed):
    """Without a BSDF density every weight descends the guide's own loss
    -w log p_guide.  With one, the lobe outputs still do (the output layer's
    lobe rows against finite differences of that loss), and the selection
    row descends -w log q, q = alpha p_guide + (1 - alpha) p_bsdf (finite
    differences of that loss; the hidden layers are checked against autograd
    with p_guide held fixed in q)."""
    G = orc.Guide
    pos, nrm, wo, om, wt = _batch(5, 1)
    pb = _bsdf_pdf(nrm, om) if mixed else None
    f = G.features(pos, nrm, wo, LO, HI)
    W = _weights(2)
    _, g = G.loss_grad(W, f, om, wt, 64, bsdf_pdf=pb, amax=AMAX)
    rng = np.random.default_rng(3)
    sel = np.arange(17408 + 40 * 64, NW)  # the selection logit's weights
    lobe_rows = np.arange(17408, 17408 + 40 * 64)
    pool = lobe_rows if mixed else np.arange(NW)
    nz = pool[np.abs(g[pool]) > 1e-4]
    checks = [(k, None) for k in rng.choice(nz, 10, replace=False)]
    if mixed:
        checks += [(k, pb) for k in rng.choice(sel[np.abs(g[sel]) > 1e-5], 4, replace=False)]
    else:
        assert not g[sel].any()
    for k, pbk in checks:
        h = np.float32(1e-3)
        Wp, Wm = W.copy(), W.copy()
        Wp[k] += h
        Wm[k] -= h
        lp, _ = G.loss_grad(Wp, f, om, wt, 64, bsdf_pdf=pbk, amax=AMAX)
        lm, _ = G.loss_grad(Wm, f, om, wt, 64, bsdf_pdf=pbk, amax=AMAX)
        fd = (lp - lm) / (float(Wp[k]) - float(Wm[k]))
        assert abs(fd - g[k]) <= 1e-5 + 1e-4 * abs(g[k]), (k, fd, g[k])


@pytest.mark.parametrize("mixed", [False, True])
def test_oracle_matches_torch_autograd(orc, mixed):
    torch = pytest.importorskip("torch")
    G = orc.Guide
    pos, nrm, wo, om, wt = _batch(7, 4)
    pb = _bsdf_pdf(nrm, om)
    f = G.features(pos, nrm, wo, LO, HI)
    W = _weights(5)
    loss_o, g_o = G.loss_grad(W, f, om, wt, 64, bsdf_pdf=pb if mixed else None, amax=AMAX)
    out_o = G.forward(W, f, 64)
    # independent model: plain torch ops in float64
    Wt = torch.tensor(W.astype(np.float64), requires_grad=True)
    shapes = [(64, 80), (64, 64), (64, 64), (64, 64), (41, 64)]
    offs = np.cumsum([0] + [a * b for a, b in shapes])
    x = torch.tensor(f)
    for l, (a, b) in enumerate(shapes):
        Wl = Wt[offs[l]:offs[l + 1]].reshape(a, b)
        x = x @ Wl.T
        if l < 4:
            x = torch.relu(x)
    out = x
    assert np.allclose(out.detach().numpy(), out_o, rtol=1e-10, atol=1e-12)
    o = out[:, :40].reshape(-1, 8, 5)
    r = o[:, :, :3]
    mu = r / torch.clamp(r.norm(dim=2, keepdim=True), min=1e-6)
    kap = torch.exp(torch.clamp(o[:, :, 3], -4.6, 6.9))
    pi = torch.softmax(o[:, :, 4], dim=1)
    w = torch.tensor(om.astype(np.float64))
    d = (mu * w[:, None, :]).sum(2)
    c = kap / (2 * np.pi * (-torch.expm1(-2 * kap)))
    p = (pi * c * torch.exp(kap * (d - 1))).sum(1)
    wtt = torch.tensor(wt.astype(np.float64))
    loss = -(wtt * torch.log(p)).sum()
    objective = loss
    if mixed:
        # the selection descends the mixture's loss with p_guide held fixed
        a = AMAX * torch.sigmoid(out[:, 40])
        pbt = torch.tensor(pb.astype(np.float64))
        loss = -(wtt * torch.log(a * p + (1 - a) * pbt)).sum()
        objective = objective - (wtt * torch.log(a * p.detach() + (1 - a) * pbt)).sum()
    objective.backward()
    assert abs(loss.item() - loss_o) <= 1e-9 * abs(loss_o)
    assert np.allclose(Wt.grad.numpy(), g_o, rtol=1e-7, atol=1e-10)


def test_vmf_mixture_is_a_density(orc):
    G = orc.Guide
    rng = np.random.default_rng(6)
    out = rng.standard_normal(41) * 1.5
    # midpoint quadrature over (cos theta, phi)
    nt, npf = 400, 400
    ct = (np.arange(nt) + 0.5) / nt * 2 - 1
    ph = (np.arange(npf) + 0.5) / npf * 2 * np.pi
    tot = 0.0
    for c in ct[::1]:
        s = np.sqrt(1 - c * c)
        for p_ in ph[::8]:
            tot += G.pdf(out, [s * np.cos(p_), s * np.sin(p_), c])
    tot *= (2.0 / nt) * (2 * np.pi / (npf / 8))
    assert abs(tot - 1.0) < 2e-2, tot


def test_bf16_mode_close_to_fp64(orc):
    G = orc.Guide
    pos, nrm, wo, _, _ = _batch(64, 8)
    f = G.features(pos, nrm, wo, LO, HI)
    W = _weights(9)
    a = G.forward(W, f, 64)
    b = G.forward(W, f, 16)
    assert np.sqrt(np.mean((a - b) ** 2)) < 0.05 * np.sqrt(np.mean(a ** 2))


# ------------------------------------------------------------------ GPU ----
@pytest.mark.gpu
def test_guide_forward_matches_oracle(ctx, orc):
    G = orc.Guide
    W = _weights(11)
    ctx.guide_set_weights(W)
    pos, nrm, wo, _, _ = _batch(1000, 12)
    got = ctx.guide_forward(pos, nrm, wo, LO, HI)
    ref = G.forward(W, G.features(pos, nrm, wo, LO, HI), 16)
    rms = np.sqrt(np.mean((got - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
    assert rms <= 1e-2, rms
    assert np.array_equal(ctx.guide_get_weights(), W)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_guide_gradient_matches_oracle(ctx, orc, mixed):
    """Without and with the BSDF density (the full sampling density's loss,
    which also trains the selection logit)."""
    G = orc.Guide
    W = _weights(13)
    ctx.guide_set_weights(W)
    pos, nrm, wo, om, wt = _batch(700, 14)
    pb = _bsdf_pdf(nrm, om) if mixed else None
    g, loss = ctx.guide_gradient(pos, nrm, wo, om, wt, LO, HI, bsdf_pdf=pb, alpha_max=AMAX)
    f = G.features(pos, nrm, wo, LO, HI)
    loss_o, g_o = G.loss_grad(W, f, om, wt, 16, bsdf_pdf=pb, amax=AMAX)
    assert abs(loss - loss_o) <= 1e-2 * abs(loss_o)
    rel = np.linalg.norm(g - g_o) / np.linalg.norm(g_o)
    cos = g @ g_o / (np.linalg.norm(g) * np.linalg.norm(g_o))
    assert rel <= 3e-2 and cos >= 0.999, (rel, cos)
    # per layer too (each has its own kernel instance), and the selection
    # logit's row of the output layer on its own
    sel = 17408 + 40 * 64
    for a, b in ((0, 5120), (5120, 9216), (9216, 13312), (13312, 17408), (17408, sel), (sel, NW)):
        if not mixed and a == sel:
            assert not g[a:b].any()
            continue
        r = np.linalg.norm(g[a:b] - g_o[a:b]) / max(np.linalg.norm(g_o[a:b]), 1e-12)
        assert r <= 5e-2, (a, r)


@pytest.mark.gpu
def test_guide_selection_bound_is_checked(ctx):
    """With BSDF densities the selection's bound alpha_max must lie in
    (0, 1); the call is refused before any launch otherwise."""
    import vermeer_gb300 as vg
    ctx.guide_init(1)
    pos, nrm, wo, om, wt = _batch(64, 3)
    pb = _bsdf_pdf(nrm, om)
    for bad in (0.0, 1.0, 1.5):
        with pytest.raises(vg.VmrError):
            ctx.guide_gradient(pos, nrm, wo, om, wt, LO, HI, bsdf_pdf=pb, alpha_max=bad)
    g, loss = ctx.guide_gradient(pos, nrm, wo, om, wt, LO, HI, bsdf_pdf=pb, alpha_max=0.5)
    assert np.isfinite(loss) and np.isfinite(g).all()


@pytest.mark.gpu
def test_guide_training_fits_a_lobe(ctx):
    """Directions drawn around one axis: Adam steps on the guide's loss make
    the mixture put its mass there."""
    ctx.guide_init(21)
    rng = np.random.default_rng(22)
    n = 4096
    pos, nrm, wo, _, _ = _batch(n, 23)
    target = np.array([0.0, 0.6, 0.8], np.float32)
    first = last = None
    for step in range(150):
        om = target[None, :] + 0.15 * rng.standard_normal((n, 3)).astype(np.float32)
        om /= np.linalg.norm(om, axis=1, keepdims=True)
        loss = ctx.guide_train_step(pos, nrm, wo, om, np.ones(n, np.float32), LO, HI, lr=3e-3)
        first = loss if first is None else first
        last = loss
    assert last < first - 2.0 * n, (first, last)
