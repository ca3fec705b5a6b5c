"""The learned part of the add proposal on the GPU: the tcgen05 forward pass
and the hand-written backward pass against numpy, and the sampler's
posterior against the plain adaptive sampler's (MH stays exact)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NPAR = 18817
F, H = 16, 128
OW1, OB1 = 0, H * F
OW2, OB2 = OB1 + H, OB1 + H + H * H
OW3, OB3 = OB2 + H, OB2 + 2 * H


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), back as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def unpack(th):
    W1 = th[OW1:OB1].reshape(H, F)
    b1 = th[OB1:OW2]
    W2 = th[OW2:OB2].reshape(H, H)
    b2 = th[OB2:OW3]
    w3 = th[OW3:OB3]
    b3 = th[OB3]
    return W1, b1, W2, b2, w3, b3


def learned_case(bmg, tmp_path, **kw):
    from bmagwa_gb300 import synth
    cfg = dict(name="plain", n=600, p=3000, chains=2, iters=60, n_rao=2)
    cfg.update(kw)
    ini = synth.make_dataset(cfg.pop("name"), str(tmp_path), **cfg)
    opt = bmg.options_from_ini(ini)
    packed, y, e = bmg.read_plink(opt)
    opt.proposal = 1  # BMG_PROPOSAL_LEARNED
    opt.learned_topk = 64
    opt.learned_every = 2
    opt.n_rao_burnin = 1000
    return opt, packed, y, e


def context(bmg, opt, packed, y, e):
    ctx = bmg.Context(opt)
    ctx.load_bed(packed)
    ctx.set_phenotypes(y)
    ctx.set_covariates(e)
    ctx.precompute()
    return ctx


def test_forward_pass_matches_numpy(bmg, tmp_path):
    opt, packed, y, e = learned_case(bmg, tmp_path)
    ctx = context(bmg, opt, packed, y, e)
    ctx.run(60, collect=False)
    th, lg, ft, tables = ctx.learned_snapshot(features=True)
    assert all(len(t[0]) > 0 for t in tables)
    W1, b1, W2, b2, w3, b3 = unpack(th)
    X = ft.reshape(-1, F)
    z1 = bf16(X).astype(np.float64) @ bf16(W1).astype(np.float64).T + b1
    h1 = bf16(np.maximum(z1, 0).astype(np.float32)).astype(np.float64)
    z2 = h1 @ bf16(W2).astype(np.float64).T + b2
    ref = np.maximum(z2, 0) @ w3 + b3
    got = lg.reshape(-1).astype(np.float64)
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)
    # FP32 accumulation order can move an activation across a bf16 rounding
    # boundary; nearly all rows agree to FP32 accuracy
    assert np.mean(err < 1e-3) > 0.995, np.sort(err)[-10:]
    assert err.max() < 5e-2
    ctx.close()


def test_backward_pass_matches_numpy(bmg, tmp_path):
    opt, packed, y, e = learned_case(bmg, tmp_path)
    ctx = context(bmg, opt, packed, y, e)
    ctx.run(40, collect=False)
    th, _, ft, _ = ctx.learned_snapshot(features=True)
    rng = np.random.default_rng(5)
    rows = np.stack([rng.integers(0, opt.n_chains, 300), rng.integers(0, opt.m_g, 300)], 1).astype(np.uint32)
    g = ctx.learned_grad(rows)
    W1, b1, W2, b2, w3, b3 = [np.asarray(a, dtype=np.float64) for a in unpack(th)]
    X = ft[rows[:, 0], rows[:, 1]].astype(np.float64)
    t = np.array([ctx.proposal(int(c))[0][int(j)] for c, j in rows])
    z1 = X @ W1.T + b1
    h1 = np.maximum(z1, 0)
    z2 = h1 @ W2.T + b2
    h2 = np.maximum(z2, 0)
    lgt = h2 @ w3 + b3
    d = (1 / (1 + np.exp(-lgt)) - t) / len(rows)
    gw3 = h2.T @ d
    gb3 = d.sum()
    dz2 = np.outer(d, w3) * (z2 > 0)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * (z1 > 0)
    gW1 = dz1.T @ X
    gb1 = dz1.sum(0)
    ref = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gw3, [gb3]])
    scale = np.abs(ref).max()
    assert scale > 0
    np.testing.assert_allclose(g, ref, rtol=1e-3, atol=1e-4 * scale)
    ctx.close()


def test_learned_sampler_targets_the_same_posterior(bmg, tmp_path):
    """Posterior inclusion probabilities (RB, averaged over chains) of the
    learned-proposal sampler agree with the plain adaptive sampler's within
    Monte Carlo error on the same data: the mixture's forward and backward
    proposal probabilities keep MH exact."""
    from bmagwa_gb300 import synth
    ini = synth.make_dataset("plain", str(tmp_path), n=400, p=40, chains=24, iters=6000, seed=3)
    pips = {}
    for mode in (0, 1):
        opt = bmg.options_from_ini(ini)
        packed, y, e = bmg.read_plink(opt)
        opt.n_rao = 5
        opt.thin = 5
        opt.n_rao_burnin = 200
        opt.proposal = mode
        opt.learned_topk = 12
        opt.learned_every = 5
        opt.learned_mix = 0.5
        ctx = context(bmg, opt, packed, y, e)
        ctx.run(6000, collect=False)
        if mode == 1:
            tables = ctx.learned_snapshot()[3]
            assert all(len(t[0]) > 0 for t in tables)
        pips[mode] = np.stack([ctx.rao(c)[0] for c in range(opt.n_chains)])
        ctx.close()
    a, b = pips[0], pips[1]
    se = np.sqrt(a.var(0, ddof=1) / len(a) + b.var(0, ddof=1) / len(b))
    diff = np.abs(a.mean(0) - b.mean(0))
    assert np.all(diff <= 5 * se + 0.02), (diff.max(), np.argmax(diff - 5 * se))
