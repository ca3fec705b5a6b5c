"""The seeded generator that stands in for the benchmark datasets: its PLINK
packing, and that its genotypes and phenotypes have the distributions the
workloads name (MAF ~ U(0.05, 0.5), Binomial(2, MAF) calls, AR(1) latent LD
with correlation 0.8 inside blocks and none across them, standardised
phenotypes from the drawn causal SNPs)."""
import numpy as np
import torch

import helpers as H
from bmagwa_gb300 import synth


def test_pack_matches_plink_layout():
    g, _ = synth.genotypes(203, 37, 0, seed=4)
    packed = synth.pack(g, chunk=8).numpy()
    assert packed.shape == (37, (203 + 3) // 4)
    assert np.array_equal(H.decode(packed.reshape(-1), 203, 37), g.numpy().astype(np.int8))
    # the unused bits of each row's last byte stay zero
    assert np.all(packed[:, -1] >> 6 == 0)


def test_independent_genotypes_follow_their_allele_frequencies():
    n, p = 20000, 200
    g, maf = synth.genotypes(n, p, 0, seed=9)
    maf = maf.numpy()
    assert maf.min() >= 0.05 and maf.max() <= 0.5
    freq = g.numpy().astype(np.float64).mean(1) / 2
    # binomial standard error of an allele frequency over 2n alleles is below 0.0025
    assert np.abs(freq - maf).max() < 0.012
    het = (g.numpy() == 1).mean(1)
    assert np.abs(het - 2 * maf * (1 - maf)).max() < 0.02


def test_ld_blocks_correlate_inside_and_not_across():
    n, p, block = 8000, 400, 50
    g, maf = synth.genotypes(n, p, block, seed=3)
    x = g.numpy().astype(np.float64)
    freq = x.mean(1) / 2
    assert np.abs(freq - maf.numpy()).max() < 0.02
    x = (x - x.mean(1, keepdims=True)) / x.std(1, keepdims=True)
    r = (x[:-1] * x[1:]).mean(1)  # correlation of neighbouring SNPs
    boundary = (np.arange(1, p) % block) == 0
    assert r[~boundary].mean() > 0.4
    assert np.abs(r[boundary]).max() < 0.05


def test_phenotype_is_standardised_and_uses_the_causal_snps():
    n, p = 5000, 300
    g, _ = synth.genotypes(n, p, 0, seed=1)
    y, idx, beta = synth.phenotype(g, 10, 0.3, 0, seed=5)
    assert y.shape == (n,) and len(idx) == 10 and len(beta) == 10
    assert abs(y.mean()) < 1e-12 and abs(y.std(ddof=1) - 1) < 1e-12
    # regressing y on the causal SNPs recovers effects proportional to beta
    x = g.numpy()[idx].astype(np.float64).T
    x = np.column_stack([np.ones(n), x])
    coef = np.linalg.lstsq(x, y, rcond=None)[0][1:]
    assert np.corrcoef(coef, beta)[0, 1] > 0.9
    y2, idx2, _ = synth.phenotype(g, (5, 100), 0.1, 0, seed=6)
    assert 5 <= len(idx2) <= 100
    y3, _, _ = synth.phenotype(g, 10, 0.3, 0, seed=5)
    assert np.array_equal(y, y3)


def test_dominance_snps_enter_through_the_heterozygote_indicator():
    n, p = 6000, 50
    g, _ = synth.genotypes(n, p, 0, seed=2)
    y, idx, beta = synth.phenotype(g, 4, 1.0, 4, seed=8)
    xa = g.numpy()[idx].astype(np.float64).T
    xh = (xa == 1).astype(np.float64)
    fit = lambda x: np.linalg.lstsq(np.column_stack([np.ones(n), x]), y, rcond=None)[1][0]
    assert fit(xh) < fit(xa)
    assert torch.is_tensor(g)
