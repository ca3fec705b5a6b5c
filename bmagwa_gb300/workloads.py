"""The synthetic workloads of the measurements and of the parity tests at the
measured sizes: their shapes, sampler settings and seeded data.

Each workload follows one configuration of the sampler's throughput study:

  plain       n = 1,000, p = 5,000, independent SNPs, additive coding,
              10 causal SNPs, one chain
  batched     n = 5,000, p = 50,000, LD blocks of 50, types A and AH,
              20 causal SNPs, 8 chains, RB every 500 iterations
  scan        n = 10,000, p = 500,000, LD blocks of 50, 30 causal SNPs,
              32 chains, the RB scan every iteration
  learned     n = 10,000, p = 200,000, LD blocks of 100, 50 causal SNPs
              (10 in dominance coding), 16 chains, learned add proposal
  phenotypes  n = 20,000, p = 1,000,000, 256 phenotypes each with its own
              missingness mask keeping 40-100 % of the individuals

The prior and sampler keys follow the reference's example configuration
(testdata/testdata.ini: e_qg = 20, var_qg = 300, nu_sigma2 = 1,
R2mode_sigma2 = 0.2, nu_tau2 = 5, s2_tau2 = 0.05, mu_alpha = 1,
max_move_size = 20).  Options are filled without loading the CUDA library
(abi.default_options), so the oracle can use them alone.
"""
import numpy as np

from . import abi

WORKLOADS = {
    "scan": dict(n=10000, p=500000, chains=32, n_rao=1, ld_block=50, causal=30, types="A"),
    "batched": dict(n=5000, p=50000, chains=8, n_rao=500, ld_block=50, causal=20, types="A,AH"),
    "plain": dict(n=1000, p=5000, chains=1, n_rao=500, ld_block=0, causal=10, types="A"),
    # the learned proposal against the plain adaptive one (inclusion ESS/s)
    "learned": dict(n=10000, p=200000, chains=16, n_rao=1, ld_block=100, causal=50, types="A,AH", dominance=10,
                    burnin=600, sample=1500),
    # many phenotypes of uneven sample size: one chain per phenotype, each
    # fitted to the individuals its missingness mask keeps (8k-20k)
    "phenotypes": dict(n=20000, p=1000000, chains=256, n_rao=1, ld_block=50, causal=(5, 100), beta_sd=0.1,
                       types="A", keep=(0.4, 1.0)),
}


def chain_seeds(seed0, chains):
    """Seed of chain c: seed0 + 1000 c (the same chain has the same seed in
    any run of the workload, whatever the chain count)."""
    return [seed0 + 1000 * c for c in range(chains)]


def options(wl, seed0, iters, chains=None):
    """Sampler options of workload wl for `iters` iterations; burn-in of the
    RB average is the first half of the run."""
    o = abi.default_options()
    o.n, o.m_g, o.m_e = wl["n"], wl["p"], 0
    types = [abi.TYPE_NAMES[t] for t in wl["types"].split(",")]
    o.n_types = len(types)
    for i, t in enumerate(sorted(types)):
        o.types[i] = t
    o.do_n_iter = iters
    o.n_rao = wl["n_rao"]
    o.thin = 1 if wl["n_rao"] < 10 else 10
    o.n_rao_burnin = max(1, iters // (2 * wl["n_rao"]))
    o.n_sample_tau2_and_missing = 10
    o.max_move_size = wl.get("max_move_size", 20)
    o.max_SNP_neighborhood_size = 20
    o.p_move_size, o.p_move_size_nbs, o.p_move_size_nbc = 0.2, 0.7, 0.25
    o.e_qg, o.var_qg, o.nu_sigma2, o.R2mode_sigma2, o.mu_alpha = 20, 300, 1, 0.2, 1
    o.inv_tau2_e_const_val, o.inv_tau2_e_val = 0.0, 0.001
    for t in range(4):
        o.nu_tau2[t], o.s2_tau2[t] = 5, 0.05
    o.max_model_size = 256
    o.graph_iters = 64
    o.quiet = 1
    abi.set_seeds(o, chain_seeds(seed0, wl["chains"] if chains is None else chains))
    return o


def make_data(wl, seed, device):
    """Packed genotypes and the phenotype (or, with wl["keep"], one
    phenotype per chain and the masks of the individuals each keeps)."""
    from . import synth
    counts, _ = synth.genotypes(wl["n"], wl["p"], wl["ld_block"], seed, device=device)
    if "keep" in wl:
        rng = np.random.default_rng(seed + 101)
        ys, masks = [], []
        for k in range(wl["chains"]):
            yk, _, _ = synth.phenotype(counts, wl["causal"], wl["beta_sd"], 0, seed + 1000 * k, device=device)
            ys.append(yk)
            masks.append((rng.random(wl["n"]) < rng.uniform(*wl["keep"])).astype(np.uint8))
        y = (np.stack(ys), np.stack(masks))
    else:
        y, _, _ = synth.phenotype(counts, wl["causal"], 0.2, wl.get("dominance", 0), seed, device=device)
    packed = synth.pack(counts).cpu().numpy().reshape(-1)
    del counts
    return packed, y


def scan_terms(types):
    """Coding rows per SNP in the scan's GEMM (A, H, D, R; AH uses A and H)."""
    rows = set()
    for t in types.split(","):
        rows |= {"A": {0}, "H": {1}, "D": {2}, "R": {3}, "AH": {0, 1}}[t]
    return len(rows)
