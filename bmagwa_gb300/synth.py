"""Seeded synthetic GWAS data of the benchmark shapes, in PLINK formats.

There is no public dataset for these workloads: genotypes, effects and
phenotypes are generated from a seed.

  independent: g_ij ~ Binomial(2, MAF_j), MAF_j ~ U(0.05, 0.5)
  ld blocks:   two haplotypes per individual, each an AR(1) latent Gaussian
               along the SNPs of a block (correlation rho), thresholded at
               the Binomial allele frequency quantile; g = allele count
  phenotype:   y = sum over causal SNPs of beta_j x_j + N(0, 1), beta ~ N(0, sd^2),
               standardised; x_j is the additive count, or the heterozygote
               indicator for SNPs drawn in dominance coding

Generation runs in torch, on the GPU when one is given, so the 1e9-byte
workloads build in seconds; the packed bytes match the .bed payload layout
(SNP-major, 4 individuals per byte, codes 00/10/11 for 0/1/2).
"""
import math
import os

import numpy as np
import torch

# the benchmark workloads (sizes of the reference's synthetic configurations)
CONFIGS = {
    "plain": dict(n=1000, p=5000, ld_block=0, causal=10, beta_sd=0.3, types="A", chains=1,
                  n_rao=500, dominance=0),
    "batched": dict(n=5000, p=50000, ld_block=50, causal=20, beta_sd=0.2, types="A,AH", chains=8,
                    n_rao=500, dominance=0),
    "scan": dict(n=10000, p=500000, ld_block=50, causal=30, beta_sd=0.2, types="A", chains=32,
                 n_rao=1, dominance=0),
    "learned": dict(n=10000, p=200000, ld_block=100, causal=50, beta_sd=0.2, types="A,AH", chains=16,
                    n_rao=1, dominance=10),
    "phenotypes": dict(n=20000, p=1000000, ld_block=50, causal=(5, 100), beta_sd=0.1, types="A",
                       chains=256, n_rao=1, dominance=0),
}


def _normal_icdf(p):
    return math.sqrt(2.0) * torch.erfinv(2.0 * p - 1.0)


def genotypes(n, p, ld_block, seed, device="cpu", rho=0.8, chunk=4096, block_group=None):
    """Allele counts (p x n, uint8) and MAFs (p,)."""
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    maf = 0.05 + 0.45 * torch.rand(p, generator=g, device=device, dtype=torch.float64)
    out = torch.empty((p, n), dtype=torch.uint8, device=device)
    thr = _normal_icdf(1.0 - maf).to(torch.float32)  # P(z > thr) = maf
    if ld_block <= 0:
        for s in range(0, p, chunk):
            e = min(p, s + chunk)
            u = torch.rand((e - s, n, 2), generator=g, device=device)
            out[s:e] = (u < maf[s:e, None, None].float()).sum(-1).to(torch.uint8)
        return out, maf
    q = math.sqrt(1.0 - rho * rho)
    nb = (p + ld_block - 1) // ld_block
    # blocks advance together: step j of every block of a group at once
    group = block_group or max(1, min(nb, (1 << 26) // max(1, 2 * n)))
    for b0 in range(0, nb, group):
        b1 = min(nb, b0 + group)
        z = torch.randn((b1 - b0, n, 2), generator=g, device=device)
        for j in range(ld_block):
            if j > 0:
                z = rho * z + q * torch.randn((b1 - b0, n, 2), generator=g, device=device)
            snps = torch.arange(b0, b1, device=device) * ld_block + j
            ok = snps < p
            if not bool(ok.any()):
                break
            snps = snps[ok]
            out[snps] = (z[ok] > thr[snps][:, None, None]).sum(-1).to(torch.uint8)
    return out, maf


def pack(counts, chunk=16384):
    """Allele counts (p x n) -> PLINK SNP-major payload (p x ceil(n/4) bytes),
    in chunks of SNPs with uint8 arithmetic (code 0 -> 00, 1 -> 10, 2 -> 11)."""
    p, n = counts.shape
    n4 = (n + 3) // 4
    out = torch.empty((p, n4), dtype=torch.uint8, device=counts.device)
    for j0 in range(0, p, chunk):
        c = counts[j0:j0 + chunk].to(torch.uint8)
        code = torch.zeros((c.shape[0], n4 * 4), dtype=torch.uint8, device=counts.device)
        code[:, :n] = (c > 0).to(torch.uint8) * 2 + (c > 1).to(torch.uint8)
        code = code.view(-1, n4, 4)
        out[j0:j0 + chunk] = code[..., 0] | (code[..., 1] << 2) | (code[..., 2] << 4) | (code[..., 3] << 6)
    return out


def phenotype(counts, causal, beta_sd, dominance, seed, device="cpu"):
    """y (n,) float64 from `causal` random SNPs; returns y, causal idx, betas."""
    p, n = counts.shape
    rng = np.random.default_rng(seed + 7)
    k = causal if isinstance(causal, int) else int(rng.integers(causal[0], causal[1] + 1))
    idx = np.sort(rng.choice(p, size=k, replace=False))
    beta = rng.normal(0.0, beta_sd, size=k)
    dom = np.zeros(k, dtype=bool)
    if dominance:
        dom[rng.choice(k, size=min(dominance, k), replace=False)] = True
    x = counts[torch.as_tensor(idx, device=counts.device)].to(torch.float64)
    xh = (x == 1).to(torch.float64)
    xe = torch.where(torch.as_tensor(dom, device=counts.device)[:, None], xh, x)
    yg = (torch.as_tensor(beta, device=counts.device)[:, None] * xe).sum(0)
    noise = torch.as_tensor(rng.normal(size=n), device=counts.device)
    y = yg + noise
    y = (y - y.mean()) / y.std()
    return y.double().cpu().numpy(), idx, beta


def write_plink(prefix, packed, y):
    packed = packed.cpu().numpy() if torch.is_tensor(packed) else packed
    with open(prefix + ".bed", "wb") as f:
        f.write(bytes([0x6C, 0x1B, 0x01]))
        f.write(np.ascontiguousarray(packed).tobytes())
    with open(prefix + ".fam", "w") as f:
        for i, v in enumerate(y):
            f.write("F%d I%d 0 0 1 %.17g\n" % (i, i, v))
    p = packed.shape[0]
    with open(prefix + ".bim", "w") as f:
        for j in range(p):
            f.write("1 rs%d 0 %d A G\n" % (j, j + 1))


INI_TEMPLATE = """; synthetic workload {name}
[datafiles]
file_fam = {prefix}.fam
file_g = {prefix}.bed
recode_g_to_minor_allele_count = 0

[sizes]
n = {n}
m_g = {p}
m_e = 0

[sampler]
type = PMV
do_n_iter = {iters}
n_rao = {n_rao}
n_rao_burnin = {burnin}
adaptation = 0
verbosity = {verbosity}
thin = {thin}
n_sample_tau2_and_missing = {nst}
delay_rejection = 0
p_move_size = 0.2
p_move_size_nbc = 0.25
p_move_size_nbs = 0.7
max_SNP_neighborhood_size = 20
adapt_p_move_size = 1
p_move_size_acpt_goal = 0
max_move_size = 20
flat_proposal_dist = 0

[thread]
n_threads = {chains}
basename = {outdir}/chain
seeds = {seeds}

[model]
types = {types}

[prior]
use_individual_tau2 = 0
type_A = 1
type_H = 1
type_D = 1
type_R = 1
type_AH = 1
e_qg = 20
var_qg = 300
R2mode_sigma2 = 0.2
nu_sigma2 = 1
nu_tau2_A = 5
s2_tau2_A = 0.05
nu_tau2_H = 5
s2_tau2_H = 0.05
mu_alpha = 1
inv_tau2_e_const_val = 0
inv_tau2_e_val = 0.001
"""


def write_ini(path, name, prefix, outdir, n, p, chains, types, n_rao, iters, thin=None, burnin=None,
              nst=10, verbosity=0, seed0=1):
    thin = thin or min(10, n_rao)
    if n_rao % thin:
        thin = 1
    burnin = burnin if burnin is not None else max(1, min(1000, iters // (2 * n_rao)))
    seeds = ",".join(str(seed0 + 1000 * c) for c in range(chains))
    txt = INI_TEMPLATE.format(name=name, prefix=prefix, outdir=outdir, n=n, p=p, iters=iters,
                              n_rao=n_rao, burnin=burnin, verbosity=verbosity, thin=thin, nst=nst,
                              chains=chains, seeds=seeds, types=types)
    with open(path, "w") as f:
        f.write(txt)
    return path


def make_dataset(name, outdir, n=None, p=None, chains=None, iters=1000, seed=1, device="cpu", **over):
    """Write a workload (PLINK files + INI) under outdir; returns the INI path."""
    cfg = dict(CONFIGS[name])
    cfg.update(over)
    n = n or cfg["n"]
    p = p or cfg["p"]
    chains = chains or cfg["chains"]
    os.makedirs(outdir, exist_ok=True)
    counts, _ = genotypes(n, p, cfg["ld_block"], seed, device=device)
    y, _, _ = phenotype(counts, cfg["causal"], cfg["beta_sd"], cfg["dominance"], seed, device=device)
    prefix = os.path.join(outdir, "data")
    write_plink(prefix, pack(counts), y)
    return write_ini(os.path.join(outdir, "run.ini"), name, prefix, outdir, n, p, chains, cfg["types"],
                     cfg["n_rao"], iters, seed0=seed)
