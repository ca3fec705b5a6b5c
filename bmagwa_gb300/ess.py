"""Effective sample size of the SNP inclusion indicators.

The reference reports no ESS.  The throughput figure "inclusion-ESS per
second" uses, per chain, the thinned trace of gamma_j (1 when SNP j is in the
model) for the SNPs whose posterior inclusion frequency lies strictly between
`lo` and `hi`, and Geyer's initial monotone sequence estimator of the
integrated autocorrelation time (Geyer 1992, "Practical Markov chain Monte
Carlo", Statist. Sci. 7:473-483):

    tau = -1 + 2 * sum_{k>=0} G_k,   G_k = rho(2k) + rho(2k+1),

summed while G_k > 0, with each G_k capped by the previous one.  ESS = T / tau.
"""
import numpy as np


def autocorr(x):
    """Normalised autocorrelation rho(0..T-1) of a 1-D series (FFT, biased)."""
    x = np.asarray(x, dtype=np.float64)
    T = len(x)
    x = x - x.mean()
    f = np.fft.rfft(x, n=2 * T)
    acov = np.fft.irfft(f * np.conj(f))[:T] / T
    if acov[0] <= 0:
        return None
    return acov / acov[0]


def ess_geyer(x):
    """ESS of one series; nan for a constant series."""
    T = len(x)
    rho = autocorr(x)
    if rho is None:
        return float("nan")
    s, prev = 0.0, np.inf
    for k in range(T // 2):
        g = rho[2 * k] + (rho[2 * k + 1] if 2 * k + 1 < T else 0.0)
        if g <= 0:
            break
        g = min(g, prev)
        s += g
        prev = g
    tau = max(-1.0 + 2.0 * s, 1.0 / T)
    return T / tau


def indicator_matrix(modelsize, loci):
    """(T, p_used) 0/1 matrix of the thinned samples and the SNP ids of its
    columns, from the trace's model sizes and flattened loci."""
    modelsize = np.asarray(modelsize, dtype=np.int64)
    loci = np.asarray(loci, dtype=np.int64)
    T = len(modelsize)
    snps = np.unique(loci)
    col = np.searchsorted(snps, loci)
    row = np.repeat(np.arange(T), modelsize)
    G = np.zeros((T, len(snps)), dtype=np.float64)
    G[row, col] = 1.0
    return G, snps


def inclusion_ess(modelsize, loci, lo=0.05, hi=0.95):
    """Per-SNP ESS of the inclusion indicators of one chain, for SNPs whose
    inclusion frequency f satisfies lo < f < hi.  Returns (snps, ess)."""
    G, snps = indicator_matrix(modelsize, loci)
    if G.shape[0] < 4 or G.shape[1] == 0:
        return np.zeros(0, dtype=np.int64), np.zeros(0)
    f = G.mean(axis=0)
    keep = (f > lo) & (f < hi)
    ess = np.array([ess_geyer(G[:, j]) for j in np.nonzero(keep)[0]])
    return snps[keep], ess


def summarize(chains, seconds):
    """chains: list of (modelsize, loci) per chain.  Returns min and median
    ESS over all (chain, SNP) pairs and the summed median ESS per second."""
    all_ess, per_chain = [], []
    for ms, lc in chains:
        _, e = inclusion_ess(ms, lc)
        e = e[np.isfinite(e)]
        if len(e):
            all_ess.append(e)
            per_chain.append(float(np.median(e)))
    if not all_ess:
        return {"snps": 0, "min": None, "median": None, "per_s": None}
    cat = np.concatenate(all_ess)
    return {"snps": int(len(cat)), "min": float(cat.min()), "median": float(np.median(cat)),
            "per_s": float(sum(per_chain) / seconds) if seconds > 0 else None}
