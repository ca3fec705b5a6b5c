"""Shared helpers of the test suite: fixtures on disk, trace comparison, and a
plain numpy restatement of the model marginal likelihood."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

INT_KEYS = ("jumpdistance", "move_type", "move_size", "modelsize", "loci", "types")
FLOAT_KEYS = ("log_likelihood", "log_prior", "sigma2", "alpha", "pve")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def materialize(z, d):
    """Write a reference fixture's input files into d; returns the INI path."""
    for key in z.files:
        if key.startswith("file_"):
            fn = key[5:].replace("_", ".", 1)
            with open(os.path.join(d, fn), "wb") as f:
                f.write(z[key].tobytes())
    os.makedirs(os.path.join(d, "out"), exist_ok=True)
    ini = z["ini"].tobytes().decode().replace("{DIR}", str(d))
    path = os.path.join(d, "run.ini")
    with open(path, "w") as f:
        f.write(ini)
    return path


def ref_chain(z, c):
    out = {}
    for key in INT_KEYS + FLOAT_KEYS + ("rao", "rao_types"):
        k = "c%d_%s" % (c, key)
        out[key] = z[k] if k in z.files else None
    return out


def compare(a, b, rtol=1e-9, keys=None, label=""):
    """Integer traces must be identical; float traces within rtol (relative)."""
    keys = keys or (INT_KEYS + FLOAT_KEYS)
    for key in keys:
        x, y = a.get(key), b.get(key)
        if x is None or y is None or (len(x) == 0 and len(y) == 0):
            continue
        assert len(x) == len(y), "%s %s: length %d vs %d" % (label, key, len(x), len(y))
        if key in INT_KEYS:
            bad = np.nonzero(np.asarray(x) != np.asarray(y))[0]
            assert len(bad) == 0, "%s %s differs first at %d (%s vs %s)" % (
                label, key, bad[0], x[bad[0]], y[bad[0]])
        else:
            x = np.asarray(x, dtype=np.float64)
            y = np.asarray(y, dtype=np.float64)
            den = np.maximum(np.abs(x), 1e-300)
            rel = np.abs(x - y) / den
            ok = (rel <= rtol) | (np.abs(x - y) <= rtol)
            assert ok.all(), "%s %s max rel diff %.3g" % (label, key, rel.max())


def decode(packed, n, p):
    """PLINK SNP-major payload -> additive genotypes (p x n), missing = -1."""
    stride = (n + 3) // 4
    b = np.asarray(packed, dtype=np.uint8).reshape(p, stride)
    codes = np.stack([(b >> (2 * k)) & 3 for k in range(4)], axis=-1).reshape(p, stride * 4)[:, :n]
    lut = np.array([0, -1, 1, 2], dtype=np.int8)
    return lut[codes]


def coding(g, term):
    """term coding of additive genotypes: A, H, D, R (missing stays -1)."""
    g = np.asarray(g)
    if term == 0:
        v = g.astype(float)
    elif term == 1:
        v = (g == 1).astype(float)
    elif term == 2:
        v = (g > 0).astype(float)
    else:
        v = (g == 2).astype(float)
    v[g < 0] = -1
    return v


def lml_numpy(X, y, inv, nu_s2_plus_yy, n_plus_nu):
    """Marginal likelihood of a linear model with prior precisions inv
    (src/model.hpp:199-237 written as plain numpy)."""
    A = X.T @ X + np.diag(inv)
    Lc = np.linalg.cholesky(A)
    v = np.linalg.solve(Lc, X.T @ y)
    s = nu_s2_plus_yy - v @ v
    return 0.5 * np.sum(np.log(inv[1:])) - np.sum(np.log(np.diag(Lc))) - 0.5 * n_plus_nu * np.log(s)


def small_opts(bg, n, p, types, **kw):
    """Options of a small test case: n individuals, p SNPs, the given effect
    types, no covariates, seed 1245; keyword arguments override fields."""
    o = bg.default_options()
    o.n, o.m_g, o.m_e = n, p, 0
    o.n_types = len(types)
    for i, t in enumerate(sorted(types)):
        o.types[i] = t
    o.do_n_iter, o.n_rao, o.n_rao_burnin, o.thin, o.n_sample_tau2_and_missing = 100, 10, 1, 10, 10
    o.e_qg, o.var_qg, o.nu_sigma2, o.s2_sigma2 = 2, 2, 1, 1
    for t in range(4):
        o.nu_tau2[t], o.s2_tau2[t] = 4, 1
    o.mu_alpha = 1
    for k, v in kw.items():
        setattr(o, k, v)
    bg.set_seeds(o, [1245])
    return o


def small_modelspace_opts(bg, n_iter, dr, seed):
    """The 7-SNP configuration of src/tests/testdata/small_modelspace_tau2.ini
    with tau2 and alpha drawn once at the start and then held (the
    n_sample_tau2_and_missing = 10^9 of onesnp_notau2.ini), so that the
    exact posterior is a sum over the 2^7 models at that fixed precision."""
    o = small_opts(bg, 30, 7, [0], e_qg=2, var_qg=2, nu_sigma2=1, s2_sigma2=0, R2mode_sigma2=0.2,
                   recode_g_to_minor_allele_count=1, inv_tau2_e_const_val=0, do_n_iter=n_iter,
                   n_rao=10, n_rao_burnin=100, thin=1, n_sample_tau2_and_missing=10 ** 9, adaptation=0,
                   delay_rejection=dr)
    o.nu_tau2[0], o.s2_tau2[0] = 3, 0.02
    bg.set_seeds(o, [seed])
    return o


def exact_pips(port):
    """Posterior inclusion probabilities of the 7 SNPs by enumerating all 2^7
    models (SamplerTestsF.SmallModelSpaceWithSharedTau2,
    src/tests/sampler_tests.hpp:348-446, with the tau2/alpha integral replaced
    by the chain's fixed precision)."""
    inv = port.inv_tau2_alpha2()[0]
    logp, _ = port.exh_modelset(list(range(7)), [0] * 7, [[inv, inv]] * 7, 0)
    w = np.exp(logp - logp.max())
    w /= w.sum()
    masks = np.arange(128)
    return np.array([w[(masks >> j) & 1 == 1].sum() for j in range(7)])
