"""GPU parity at the sizes the throughput measurements run, and at the edge
of the tensor-core scan's exactness argument.

The tensor-core scan multiplies 0/1/2 genotype codings by balanced base-256
digits of the fixed-point residual (bf16, exact) and accumulates in FP32:
every product has magnitude <= 2 x 128 = 256, so every partial sum of n
products stays below 2^24 -- an exact FP32 integer -- while n < 65,536.  The
SIMT scan forms the same x'r as an exact int64, so the two must agree bit for
bit.  These tests check that:
  - at the `scan` workload's shape (n = 10,000, 32 chains: one N tile of
    192 columns) with the workload's own generator;
  - at n = 65,000 with residual digits of magnitude 127 in every low limb,
    so that the limb sums reach 2 x 127 x 65,000 = 16,510,000, within 2 % of
    2^24;
  - with 48 masked phenotypes (two N tiles);
and that the GPU chains equal the oracle's (RaoBlackwellizer and the moves,
src/sampler.cpp:32-261, src/sampler.hpp:899-1418) on the full `scan` workload
(n = 10,000, p = 500,000, 32 chains on the GPU, two of them on the oracle) and
on the `batched` workload (n = 5,000, p = 50,000, A and AH, LD blocks,
8 chains, two RB steps)."""
import numpy as np
import pytest

import helpers as H
from test_gpu_parity import RTOL

pytestmark = pytest.mark.gpu


def _ctx(bmg, opt, packed, y, masks=None):
    ctx = bmg.Context(opt)
    ctx.load_bed(packed)
    if masks is None:
        ctx.set_phenotypes(y)
    else:
        ctx.set_phenotypes(y, masks)
    ctx.set_covariates(None)
    ctx.precompute()
    return ctx


def _pack_codes(G):
    """p x n matrix of additive genotypes (0, 1, 2) -> PLINK SNP-major payload."""
    import torch
    from bmagwa_gb300 import synth
    return synth.pack(torch.as_tensor(np.ascontiguousarray(G, dtype=np.uint8))).numpy().reshape(-1)


def test_tc_scan_bitwise_at_the_scan_workload_shape(bmg, monkeypatch):
    """n = 10,000, 32 chains in one N tile (192 columns = 32 chains x 6
    limbs), p = 50,000 SNPs of the `scan` workload's LD-block generator: the
    tensor-core scan's in-loop posteriors and every trace equal the SIMT
    scan's bit for bit after 6 iterations with an RB scan each."""
    from bmagwa_gb300 import workloads
    wl = dict(workloads.WORKLOADS["scan"], p=50000)
    packed, y = workloads.make_data(wl, 1, "cuda")
    res = {}
    for scan, variant in ((1, None), (0, "0"), (0, "6")):
        if variant is None:
            monkeypatch.delenv("BMG_SCAN_VARIANT", raising=False)
        else:
            monkeypatch.setenv("BMG_SCAN_VARIANT", variant)
        opt = workloads.options(wl, 1, 6)
        opt.scan_impl = scan
        opt.scan_limbs = 6
        ctx = _ctx(bmg, opt, packed, y)
        col = ctx.run(6)
        if variant == "0":
            assert "1/1" in ctx.scan_shape()[1]  # all 32 chains in one N tile
        res[(scan, variant)] = ([col.chain(c) for c in range(32)], [ctx.last_scan(c)[0] for c in range(32)],
                                [ctx.rao(c)[0] for c in range(32)])
        ctx.close()
    ref = res[(1, None)]
    for key, got in res.items():
        for c in range(32):
            H.compare(ref[0][c], got[0][c], rtol=0.0, label="%s chain %d" % (key, c))
            np.testing.assert_array_equal(ref[1][c], got[1][c], err_msg="%s chain %d" % (key, c))
            np.testing.assert_array_equal(ref[2][c], got[2][c], err_msg="%s chain %d" % (key, c))


def _worst_case_data(n, p, seed, two_valued, limbs=6):
    """Genotypes with long runs of code 2 and a phenotype whose fixed-point
    residual has the digit 127 (or -127) in every limb below the top one.

    The scan runs against zero fitted values (bmg_scan_yhat), so its residual
    is y itself, at the scale 2^(8 L - 4) for L limbs and max |y| in (1, 2]
    (2^44 for six limbs).  y = v + k/16 with v = 1 + 0x7F...7F / 2^(8 L - 4)
    (L - 1 bytes 0x7F) puts 0x7F in every byte of the low 8 (L - 1) bits of
    every individual's residual: the low limbs are 127 everywhere and only
    the top limb varies (16 + k).  two_valued gives the second half of the
    individuals -y instead (digits -127)."""
    rng = np.random.default_rng(seed)
    v = 1.0 + float(int("7F" * (limbs - 1), 16)) / 2.0 ** (8 * limbs - 4)
    k = rng.integers(-3, 4, n)
    y = v + k / 16.0
    sign = np.ones(n)
    if two_valued:
        sign[n // 2:] = -1.0
        y = y * sign
    G = np.zeros((p, n), dtype=np.uint8)
    for j in range(p):
        kind = j % 4
        if kind == 0:    # all 2 but a few individuals
            G[j] = 2
            G[j, rng.integers(0, n, 8)] = 0
        elif kind == 1:  # 2 on the positive half, else 0 (all 2 when one-signed)
            G[j] = np.where(sign > 0, 2, 0)
            G[j, rng.integers(0, n, 40)] = 1
        elif kind == 2:  # mostly 2
            G[j] = np.where(rng.random(n) < 0.97, 2, rng.integers(0, 2, n))
        else:            # ordinary allele frequencies
            G[j] = rng.binomial(2, rng.uniform(0.05, 0.5), n)
    return _pack_codes(G), y


@pytest.mark.parametrize("limbs", [5, 6])
@pytest.mark.parametrize("two_valued", [False, True], ids=["one_signed", "two_valued"])
def test_tc_scan_exact_near_the_fp32_bound(bmg, oracle, two_valued, limbs):
    """n = 65,000 (the tensor-core scan takes n below 65,536): with digits of
    magnitude 127 in every low limb, the FP32 partial sums over a column of
    2s reach 2 x 127 x 65,000 = 16,510,000 (2^24 = 16,777,216) for the
    one-signed phenotype and 8.3 million for the two-valued one.  The
    tensor-core scan equals the SIMT scan (exact int64) bit for bit, and both
    equal the oracle's FP64 scan (RaoBlackwellizer::p_raoblackwell with the
    same fitted values and sigma2) to 1e-9."""
    from bmagwa_gb300 import workloads
    n, p = 65000, 512
    packed, y = _worst_case_data(n, p, 3, two_valued, limbs)
    wl = dict(workloads.WORKLOADS["plain"], n=n, p=p, chains=2, n_rao=1)
    zero = np.zeros(n)
    out = {}
    for scan in (1, 0):
        opt = workloads.options(wl, 5, 1)
        opt.scan_impl = scan
        opt.scan_limbs = limbs
        ctx = _ctx(bmg, opt, packed, y)
        out[scan] = ctx.scan_yhat(zero, 1.0)
        ctx.close()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert np.all(np.isfinite(out[0][0]))
    opt = workloads.options(wl, 5, 1)
    port = oracle.Port(opt, packed, y)
    for c in range(2):
        ref, _ = port.scan_yhat(zero, 1.0, c)
        np.testing.assert_allclose(out[0][0][c], ref, rtol=1e-9, atol=1e-13)


def test_two_n_tiles_of_masked_phenotypes(bmg, oracle, tmp_path):
    """48 phenotypes with masks at n = 8,200: more chains than one N tile
    holds (42 x 6 limbs = 252 of 256 columns), so the scan runs two N tiles.
    Every chain equals the SIMT scan's bit for bit, and the first and last
    phenotype equal the oracle run on their subset .bed files."""
    import torch
    from bmagwa_gb300 import synth, workloads
    n, p, K, iters = 8200, 2500, 48, 40
    wl = dict(workloads.WORKLOADS["plain"], n=n, p=p, chains=K, n_rao=2, ld_block=50)
    counts, _ = synth.genotypes(n, p, 50, 7, device="cuda")
    rng = np.random.default_rng(8)
    ys = []
    for k in range(K):
        yk, _, _ = synth.phenotype(counts, 5 + k % 7, 0.3, 0, 100 + k, device="cuda")
        ys.append(yk)
    Y = np.stack(ys)
    masks = (rng.random((K, n)) < rng.uniform(0.5, 1.0, (K, 1))).astype(np.uint8)
    packed = synth.pack(counts).cpu().numpy().reshape(-1)
    G = counts.cpu().numpy()
    del counts
    res = {}
    for scan in (1, 0):
        opt = workloads.options(wl, 3, iters)
        opt.scan_impl = scan
        opt.scan_limbs = 6  # 42 chains of 6 limbs fill one N tile
        opt.adapt_p_move_size = 0  # early tuning ties break on last bits of exp
        ctx = _ctx(bmg, opt, packed, Y, masks)
        col = ctx.run(iters)
        res[scan] = ([col.chain(c) for c in range(K)], [ctx.last_scan(c)[0] for c in range(K)],
                     [ctx.rao(c)[0] for c in range(K)])
        ctx.close()
    for c in range(K):
        H.compare(res[1][0][c], res[0][0][c], rtol=0.0, label="phenotype %d" % c)
        np.testing.assert_array_equal(res[1][1][c], res[0][1][c])
    for k in (0, K - 1):
        keep = np.nonzero(masks[k])[0]
        pk = synth.pack(torch.as_tensor(G[:, keep])).numpy().reshape(-1)
        ok = workloads.options(dict(wl, n=len(keep), chains=1), 3 + 1000 * k, iters)
        ok.adapt_p_move_size = 0
        port = oracle.Port(ok, pk, Y[k][keep])
        colp = port.run(iters)
        H.compare(colp.chain(0), res[0][0][k], rtol=RTOL, label="phenotype %d vs oracle" % k)
        np.testing.assert_allclose(res[0][2][k], port.rao(0)[0], rtol=RTOL, atol=1e-12)


@pytest.mark.parametrize("name,iters,oracle_chains", [("scan", 4, 2), ("batched", 1000, 8)])
def test_gpu_matches_oracle_at_the_measured_workloads(bmg, oracle, name, iters, oracle_chains):
    """The workloads the throughput is measured on, at full size: the GPU
    runs all chains of the workload and the oracle the first `oracle_chains`
    of them (same seeds); their traces and Rao-Blackwellised posteriors
    agree (integers exactly, floats to 1e-9)."""
    from bmagwa_gb300 import workloads
    wl = workloads.WORKLOADS[name]
    packed, y = workloads.make_data(wl, 1, "cuda")
    opt = workloads.options(wl, 1, iters)
    ctx = _ctx(bmg, opt, packed, y)
    colg = ctx.run(iters)
    rao_g = [ctx.rao(c)[0] for c in range(oracle_chains)]
    ctx.close()
    ok = workloads.options(wl, 1, iters, chains=oracle_chains)
    port = oracle.Port(ok, packed, y)
    colp = port.run(iters, threads=oracle_chains)
    for c in range(oracle_chains):
        H.compare(colp.chain(c), colg.chain(c), rtol=RTOL, label="%s chain %d" % (name, c))
        np.testing.assert_allclose(rao_g[c], port.rao(c)[0], rtol=RTOL, atol=1e-12)


@pytest.mark.parametrize("n", [70000, 140000])
def test_tc_scan_beyond_65536_individuals(bmg, oracle, n):
    """Above 65,535 individuals the tensor-core scan closes its FP32
    accumulator every 65,280 individuals (a K segment) and adds the
    segments' exact integers in int64: two and three segments here.  The
    traces and in-loop posteriors equal the SIMT scan's bit for bit and the
    oracle's chain to 1e-9."""
    from bmagwa_gb300 import synth, workloads
    p, iters = 1200, 12
    wl = dict(workloads.WORKLOADS["plain"], n=n, p=p, chains=2, n_rao=2, ld_block=50)
    counts, _ = synth.genotypes(n, p, 50, 17, device="cuda")
    y, _, _ = synth.phenotype(counts, 8, 0.3, 0, 17, device="cuda")
    packed = synth.pack(counts).cpu().numpy().reshape(-1)
    del counts
    res = {}
    for scan in (1, 0):
        opt = workloads.options(wl, 7, iters)
        opt.scan_impl = scan
        opt.adapt_p_move_size = 0
        ctx = _ctx(bmg, opt, packed, y)
        col = ctx.run(iters)
        res[scan] = ([col.chain(c) for c in range(2)], [ctx.last_scan(c)[0] for c in range(2)],
                     [ctx.rao(c)[0] for c in range(2)])
        ctx.close()
    for c in range(2):
        H.compare(res[1][0][c], res[0][0][c], rtol=0.0, label="chain %d" % c)
        np.testing.assert_array_equal(res[1][1][c], res[0][1][c])
    opt = workloads.options(wl, 7, iters)
    opt.adapt_p_move_size = 0
    port = oracle.Port(opt, packed, y)
    colp = port.run(iters, threads=2)
    for c in range(2):
        H.compare(colp.chain(c), res[0][0][c], rtol=RTOL, label="oracle chain %d" % c)
        np.testing.assert_allclose(res[0][2][c], port.rao(c)[0], rtol=RTOL, atol=1e-12)
