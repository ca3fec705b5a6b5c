"""The CPU oracle against the reference's known answers and traces.

The oracle (oracle/port) is what every GPU parity test compares with, so it is
pinned first: against the golden vectors of the reference's own tests
(src/tests/*_tests.hpp) and against traces of the reference itself (the
fixtures of tests/golden, made by tests/golden/make_golden.py)."""
import ctypes as C
import math

import numpy as np
import pytest

import helpers as H


small_opts = H.small_opts


def test_decode_known_answers(bmg, oracle):
    """DataTests.LoadAndHandlePlinkData{NoMissing,WithMissing} (src/tests/data_tests.hpp:30-194)."""
    z = H.golden("data_tests")
    for bed, fam, gold, n, p in (("small_bed", "small_fam", "small_genotypes", 30, 7),
                                 ("plink_bed", "plink_fam", "plink_genotypes", 5, 10)):
        packed = z[bed][3:]
        g = z[gold]
        o = small_opts(bmg, n, p, [0])
        port = oracle.Port(o, packed, np.zeros(n) + np.arange(n) * 0.1)
        for j in range(p):
            for term in range(4):
                assert np.array_equal(port.genotypes(term, j), H.coding(g[j], term)), (bed, j, term)
        assert np.array_equal(H.decode(packed, n, p), g)


def test_phenotypes_known_answer(bmg, tmp_path):
    """The .fam phenotypes of small_modelspace (src/tests/data_tests.hpp:44-75) via the product reader."""
    z = H.golden("data_tests")
    (tmp_path / "d.bed").write_bytes(z["small_bed"].tobytes())
    (tmp_path / "d.fam").write_bytes(z["small_fam"].tobytes())
    o = small_opts(bmg, 30, 7, [0])
    bmg.abi.set_path(o, "file_fam", str(tmp_path / "d.fam"))
    bmg.abi.set_path(o, "file_g", str(tmp_path / "d.bed"))
    packed, y, _ = bmg.read_plink(o)
    assert np.array_equal(y, z["small_y"])
    assert np.array_equal(packed, z["small_bed"][3:])


@pytest.mark.parametrize("types", [[0], [0, 4], [0, 1, 2, 3, 4]])
def test_precomputed_covariances(bmg, oracle, types):
    """PrecomputedSNPCovariancesTests (src/tests/precomputed_snp_covariances_tests.hpp:30-150)."""
    z = H.golden("data_tests")
    packed, n, p = z["plink_bed"][3:], 5, 10
    o = small_opts(bmg, n, p, types)
    port = oracle.Port(o, packed, np.linspace(-1, 1, n))
    xx = port.precomputed()
    g = H.decode(packed, n, p).astype(float)
    g[g < 0] = 0  # missing values enter the precomputation as 0
    terms = sorted({t for ty in types for t in ((0, 1) if ty == 4 else (ty,))})
    for j in range(p):
        col = 0
        for t in terms:
            x = H.coding(g[j], t)
            assert xx[j, col] == pytest.approx(x.sum(), abs=1e-12)
            assert xx[j, col + 1] == pytest.approx(x @ x - x.sum() ** 2 / n, abs=1e-10)
            col += 2
        if 4 in types:
            a, h = H.coding(g[j], 0), H.coding(g[j], 1)
            assert xx[j, -1] == pytest.approx(a @ h - a.sum() * h.sum() / n, abs=1e-10)


def test_lml_known_answer(bmg, oracle):
    """ModelTests.LikelihoodComputation (src/tests/model_tests.hpp:36-90): hand-computed LMLs."""
    z = H.golden("data_tests")
    packed, n = z["plink_bed"][3:], 5
    fam = z["plink_fam"].tobytes().decode().split()
    y = np.array([float(fam[6 * i + 5]) for i in range(n)])
    o = small_opts(bmg, n, 10, [0, 4], e_qg=2, var_qg=4, nu_sigma2=4, s2_sigma2=1, mu_alpha=2,
                   inv_tau2_e_const_val=0)
    port = oracle.Port(o, packed, y)
    tau2 = 4.0 * 1.0 / (4.0 - 2.0)
    inv = 1.0 / (2.0 * 2.0 * tau2)
    lml = port.model_lml([1, 5], [0, 1], [[inv, inv], [inv, inv]])
    nu_s, s2_s = 4.0, 1.0
    syy1 = 0.58 - 0.51670588235294123702
    exp1 = -0.5 * math.log(tau2) - 0.5 * math.log(4.0 * 10.0 + 5.0 / tau2) \
        - 0.5 * (nu_s + n) * math.log(nu_s * s2_s + syy1)
    syy2 = 0.58 - 0.56537856592135671274
    exp2 = -0.5 * 3.0 * math.log(tau2) - 0.5 * math.log(810.62499999999954525265) \
        - 0.5 * (nu_s + n) * math.log(nu_s * s2_s + syy2)
    assert lml[0] == pytest.approx(exp1, abs=1e-8)
    assert lml[1] == pytest.approx(exp2, abs=1e-8)


def test_lml_matches_numpy(bmg, oracle):
    """Incremental Cholesky LML (src/model.hpp:432-506) equals a direct dense computation."""
    rng = np.random.default_rng(3)
    n, p = 80, 40
    g = rng.integers(0, 3, size=(p, n))
    code = np.where(g == 0, 0, np.where(g == 1, 2, 3)).astype(np.uint8)
    pad = np.zeros((p, (n + 3) // 4 * 4), dtype=np.uint8)
    pad[:, :n] = code
    pad = pad.reshape(p, -1, 4)
    packed = (pad[..., 0] | pad[..., 1] << 2 | pad[..., 2] << 4 | pad[..., 3] << 6).astype(np.uint8)
    y = rng.normal(size=n)
    o = small_opts(bmg, n, p, [0, 4], nu_sigma2=2, s2_sigma2=0.7, inv_tau2_e_const_val=0.01)
    port = oracle.Port(o, packed.reshape(-1), y)
    snps = [3, 17, 5, 30, 22]
    tinds = [0, 1, 0, 1, 0]
    invs = [[0.5, 0.25], [0.3, 0.4], [0.7, 0.7], [0.2, 0.9], [1.1, 1.1]]
    lml = port.model_lml(snps, tinds, invs)
    cols, precs = [np.ones(n)], [0.01]
    for step, (s, t, iv) in enumerate(zip(snps, tinds, invs)):
        cols.append(H.coding(g[s], 0))
        precs.append(iv[0])
        if t == 1:
            cols.append(H.coding(g[s], 1))
            precs.append(iv[1])
        X = np.stack(cols, 1)
        exp = H.lml_numpy(X, y, np.array(precs), 2 * 0.7 + y @ y, n + 2)
        assert lml[step] == pytest.approx(exp, rel=1e-11)


def test_lml_after_removal_matches_numpy(bmg, oracle):
    """Removing each term of a 7-term model (A and AH columns) by the Givens
    downdate (src/model.hpp:270-312,508-556; the reference's CholeskyDowndate
    test, src/tests/symmmatrix_tests.hpp:106-142, at the model level) gives the
    dense numpy LML of the model without it."""
    rng = np.random.default_rng(17)
    n, p = 70, 25
    g = rng.integers(0, 3, size=(p, n))
    code = np.where(g == 0, 0, np.where(g == 1, 2, 3)).astype(np.uint8)
    pad = np.zeros((p, (n + 3) // 4 * 4), dtype=np.uint8)
    pad[:, :n] = code
    pad = pad.reshape(p, -1, 4)
    packed = (pad[..., 0] | pad[..., 1] << 2 | pad[..., 2] << 4 | pad[..., 3] << 6).astype(np.uint8)
    y = rng.normal(size=n)
    o = small_opts(bmg, n, p, [0, 4], nu_sigma2=2, s2_sigma2=0.7, inv_tau2_e_const_val=0.01)
    port = oracle.Port(o, packed.reshape(-1), y)
    snps = [4, 19, 7, 12, 0, 23, 9]
    tinds = [1, 0, 1, 0, 0, 1, 0]
    invs = [[0.4 + 0.1 * i, 0.8 - 0.07 * i] for i in range(len(snps))]
    for rem in range(len(snps)):
        got = port.model_lml_remove(snps, tinds, invs, rem)
        cols, precs = [np.ones(n)], [0.01]
        for k in range(len(snps)):
            if k == rem:
                continue
            cols.append(H.coding(g[snps[k]], 0))
            precs.append(invs[k][0])
            if tinds[k] == 1:
                cols.append(H.coding(g[snps[k]], 1))
                precs.append(invs[k][1])
        exp = H.lml_numpy(np.stack(cols, 1), y, np.array(precs), 2 * 0.7 + y @ y, n + 2)
        assert got == pytest.approx(exp, rel=1e-11), rem


@pytest.mark.parametrize("terms,const_loci", [
    ([(0, 0), (1, 1), (2, 0), (3, 0), (4, 1)], 0),
    ([(0, 1), (1, 0), (2, 0), (3, 1), (4, 0), (5, 0), (6, 0), (7, 0)], 2),
])
def test_exhaustive_modelset_known_answer(bmg, oracle, terms, const_loci):
    """ModelTests.ExhaustiveComputation{,WithConstLoci} (src/tests/model_tests.hpp:92-235):
    every sub-model the delayed-rejection enumeration visits by adds and left
    moves has the log probability of the same model built from scratch."""
    z = H.golden("data_tests")
    packed, n = z["plink_bed"][3:], 5
    fam = z["plink_fam"].tobytes().decode().split()
    y = np.array([float(fam[6 * i + 5]) for i in range(n)])
    o = small_opts(bmg, n, 10, [0, 4], e_qg=2, var_qg=4, nu_sigma2=4, s2_sigma2=1, mu_alpha=2,
                   inv_tau2_e_const_val=0)
    port = oracle.Port(o, packed, y)
    inv = 1.0 / (2.0 * 2.0 * (4.0 * 1.0 / (4.0 - 2.0)))
    snps, tinds = zip(*terms)
    exh, direct = port.exh_modelset(snps, tinds, [[inv, inv]] * len(terms), const_loci)
    assert len(exh) == 1 << (len(terms) - const_loci)
    assert np.all(np.isfinite(exh))
    np.testing.assert_allclose(exh, direct, rtol=0, atol=1e-10)


def test_exhaustive_proposal_probabilities_known_answer(oracle):
    """SamplerTests.ExhProposals (src/tests/sampler_tests.hpp:611-700): SNPs 1
    and 2 are in the model, the move {+0, -2, +3} was proposed and SNP 1 stays;
    each of the 8 sub-models gets the probability of proposing it from the
    model with only SNP 1 (adds in order, removals in reverse, a factor 1/2
    while both adds and removes are possible)."""
    qa = [0.3, 0.4, 0.5, 0.6]
    qr = [0.7, 0.6, 0.5, 0.4]
    out = oracle.exh_proposal_probs([0, 2, 1], [0.3, 0.5, 0.6], [0.7, 0.5, 0.4], z_add=0.3 + 0.5 + 0.6,
                                    z_rem=0.6, const_loci=1, m_g=4)
    lh = math.log(0.5)
    lg = math.log
    expect = [
        lg(qa[0] / (qa[0] + qa[2] + qa[3])) + lh + lg(qa[2] / (qa[2] + qa[3])) + lh + lh,
        lg(qr[0] / (qr[0] + qr[1])) + lh + lg(qa[2] / (qa[2] + qa[3])) + lh + lh,
        lg(qa[0] / (qa[0] + qa[2])) + lh + lh + lg(qr[3] / (qr[1] + qr[3])),
        lg(qr[3] / (qr[0] + qr[1] + qr[3])) + lh + lh + lg(qr[0] / (qr[1] + qr[0])),
        lg(qa[0] / (qa[0] + qa[3])) + lh + lg(qr[2] / (qr[1] + qr[2])) + lh + lh,
        lg(qr[2] / (qr[0] + qr[1] + qr[2])) + lh + lg(qr[0] / (qr[1] + qr[0])) + lh + lh,
        lh + lg(qr[3] / (qr[3] + qr[1] + qr[2])) + lg(qr[2] / (qr[1] + qr[2])),
        lg(qr[3] / (qr[0] + qr[3] + qr[1] + qr[2])) + lg(qr[2] / (qr[0] + qr[1] + qr[2]))
        + lg(qr[0] / (qr[0] + qr[1])),
    ]
    np.testing.assert_allclose(out, expect, rtol=0, atol=1e-10)


def test_exhaustive_modelset_matches_numpy(bmg, oracle):
    """The enumeration over 8 terms with 3 kept, on sampled genotypes, against
    a dense numpy LML plus the beta-binomial/Dirichlet prior change of each
    added term (src/prior.hpp:144-150, :273-290)."""
    rng = np.random.default_rng(5)
    n, p = 90, 30
    g = rng.integers(0, 3, size=(p, n))
    code = np.where(g == 0, 0, np.where(g == 1, 2, 3)).astype(np.uint8)
    pad = np.zeros((p, (n + 3) // 4 * 4), dtype=np.uint8)
    pad[:, :n] = code
    pad = pad.reshape(p, -1, 4)
    packed = (pad[..., 0] | pad[..., 1] << 2 | pad[..., 2] << 4 | pad[..., 3] << 6).astype(np.uint8)
    y = rng.normal(size=n)
    o = small_opts(bmg, n, p, [0, 4], e_qg=3, var_qg=4, nu_sigma2=2, s2_sigma2=0.7,
                   inv_tau2_e_const_val=0.01)
    tp = [o.types_prior[0], o.types_prior[4]]
    port = oracle.Port(o, packed.reshape(-1), y)
    snps = [3, 17, 5, 29, 22, 8, 11, 0, 14, 26, 19]
    tinds = [0, 1, 0, 1, 0, 0, 1, 0, 1, 0, 0]
    invs = [[0.3 + 0.1 * i, 0.9 - 0.05 * i] for i in range(len(snps))]
    const = 3
    exh, direct = port.exh_modelset(snps, tinds, invs, const)
    np.testing.assert_allclose(exh, direct, rtol=0, atol=1e-9)
    zq = (4 - 3 * (1 - 3)) / ((p - 1) * 3)
    ga = (zq - 1) / (1 - p * zq / 3)
    gb = (p / 3 - 1) * ga
    nm = len(snps) - const
    for mask in range(1 << nm):
        keep = list(range(const)) + [const + j for j in range(nm) if (mask >> j) & 1]
        cols, precs = [np.ones(n)], [0.01]
        for k in keep:
            cols.append(H.coding(g[snps[k]], 0))
            precs.append(invs[k][0])
            if tinds[k] == 1:
                cols.append(H.coding(g[snps[k]], 1))
                precs.append(invs[k][1])
        lml = H.lml_numpy(np.stack(cols, 1), y, np.array(precs), 2 * 0.7 + y @ y, n + 2)
        ns = [sum(1 for k in range(const) if tinds[k] == t) for t in (0, 1)]
        nl, lp = const, 0.0
        for k in keep[const:]:
            t = tinds[k]
            lp += (math.log(ga + nl) - math.log(gb + p - nl - 1)) + \
                  (math.log(tp[t] + ns[t]) - math.log(tp[0] + tp[1] + nl))
            ns[t] += 1
            nl += 1
        assert exh[mask] == pytest.approx(lml + lp, rel=1e-10, abs=1e-9), mask


@pytest.mark.parametrize("dr", [0, 20])
def test_sampler_matches_exact_posterior(bmg, oracle, dr):
    """The Rao-Blackwellised inclusion probabilities of a 200k-iteration chain
    equal the exact posterior within 0.005; the visit frequencies within 0.03.
    The frequencies carry a bias of the reference's own sampler: its
    neighbourhood moves (swap and state change, src/sampler.hpp:1300-1345)
    reflect at the ends of the SNP range without a proposal ratio, which in a
    7-SNP space puts the end SNPs about 0.017 below the exact value (with
    add/remove moves alone the frequencies agree within 0.003)."""
    z = H.golden("data_tests")
    packed, y = z["small_bed"][3:], z["small_y"]
    n_iter = 200000
    o = H.small_modelspace_opts(bmg, n_iter, dr, 1245)
    port = oracle.Port(o, packed, y)
    col = port.run(n_iter)
    pip = H.exact_pips(port)
    rao, _ = port.rao()
    np.testing.assert_allclose(rao, pip, rtol=0, atol=0.005)
    c = col.chain(0)
    ms, loci = c["modelsize"], c["loci"]
    inc = np.zeros((len(ms), 7))
    inc[np.repeat(np.arange(len(ms)), ms), loci] = 1
    np.testing.assert_allclose(inc[1000:].mean(0), pip, rtol=0, atol=0.03)


def test_rb_closed_form(bmg, oracle):
    """RaoBlackwellizerTests.EmptyCurrentModel (src/tests/raoblackwellizer_tests.hpp:31-93)."""
    z = H.golden("data_tests")
    packed, n, p = z["small_bed"][3:], 30, 7
    y = z["small_y"]
    o = small_opts(bmg, n, p, [0], e_qg=2, var_qg=2, nu_sigma2=1, s2_sigma2=0, R2mode_sigma2=0.2,
                   recode_g_to_minor_allele_count=1, inv_tau2_e_const_val=0)
    o.nu_tau2[0], o.s2_tau2[0] = 3, 0.02
    port = oracle.Port(o, packed, y)
    sigma2 = 0.7318
    pr, _ = port.scan_yhat(np.zeros(n), sigma2)
    # recoded genotypes, shared tau2 at its prior initialisation, alpha = 1
    g = H.decode(packed, n, p)
    freq = g.sum(1) / (2.0 * n)
    g = np.where(freq[:, None] > 0.5, np.where(g == 0, 2, np.where(g == 2, 0, g)), g).astype(float)
    tau2 = 3 * 0.02 / max(0.1, 3 - 2)
    inv = 1.0 / tau2
    # beta-binomial hyper-parameters (src/prior.hpp:273-290) and the add change (:144-150)
    z_ = (2 - 2 * (1 - 2)) / ((p - 1) * 2)
    ga = (z_ - 1) / (1 - p * z_ / 2)
    gb = (p / 2 - 1) * ga
    lmp = (math.log(ga) - math.log(gb + p - 1)) + (math.log(1.0) - math.log(1.0))
    for j in range(p):
        x = g[j]
        xx, yx, xs, rs = x @ x, y @ x, x.sum(), y.sum()
        det = n * (xx + inv) - xs * xs
        rxxr = (rs * rs * (xx + inv) - 2.0 * yx * rs * xs + yx * yx * n) / det
        e = math.exp(0.5 * (math.log(n) - math.log(det)) + 0.5 * math.log(inv)
                     - 0.5 * (rs * rs / n - rxxr) / sigma2 + lmp)
        assert pr[j] == pytest.approx(e / (1 + e), abs=1e-10)


@pytest.mark.parametrize("name", ["small", "small_types", "example", "example_types", "small_dr", "example_dr",
                                  "small_types_dr", "small_types_missing", "example_missing", "small_flat",
                                  "example_flat", "small_types_dr_missing", "example_large",
                                  "example_types_indiv"])
def test_oracle_matches_reference_traces(bmg, oracle, tmp_path, name):
    """The oracle reproduces the compiled reference's traces bit for bit (the
    *_dr cases with delayed rejection on, the *_missing cases with missing
    genotype calls imputed and Gibbs-updated, the *_flat cases with a flat
    proposal, raw genotypes and the beta trace)."""
    z = H.golden("ref_" + name)
    ini = H.materialize(z, tmp_path)
    opt = bmg.options_from_ini(ini)
    packed, y, e = bmg.read_plink(opt)
    port = oracle.Port(opt, packed, y, e)
    col = port.run(opt.do_n_iter)
    for c in range(opt.n_chains):
        ref = H.ref_chain(z, c)
        H.compare(ref, col.chain(c), rtol=0.0, label="%s chain %d" % (name, c))
        if "c%d_beta" % c in z.files:
            assert np.array_equal(col.chain(c)["beta"], z["c%d_beta" % c]), "%s chain %d beta" % (name, c)
        rao, raot = port.rao(c)
        assert np.array_equal(rao, ref["rao"])
        if raot is not None:
            assert np.array_equal(raot.reshape(-1), ref["rao_types"])


def test_schur_scan_matches_dense_lml(bmg, oracle):
    """The oracle's per-SNP Schur scan (update_likelihood_on_add's formulas on
    each candidate column) equals LML(model + column) - LML(model) computed
    densely with numpy, for a chain state reached by sampling."""
    rng = np.random.default_rng(11)
    n, p = 120, 60
    g = rng.integers(0, 3, size=(p, n))
    code = np.where(g == 0, 0, np.where(g == 1, 2, 3)).astype(np.uint8)
    pad = np.zeros((p, (n + 3) // 4 * 4), dtype=np.uint8)
    pad[:, :n] = code
    pad = pad.reshape(p, -1, 4)
    packed = (pad[..., 0] | pad[..., 1] << 2 | pad[..., 2] << 4 | pad[..., 3] << 6).astype(np.uint8)
    y = 0.8 * H.coding(g[7], 0) - 0.6 * H.coding(g[21], 0) + rng.normal(size=n)
    o = small_opts(bmg, n, p, [0], nu_sigma2=2, s2_sigma2=0.7, inv_tau2_e_const_val=0.01)
    port = oracle.Port(o, packed.reshape(-1), y)
    port.run(40)
    st, loci, tinds = port.state(0)
    assert len(loci) >= 1
    dl, itv = port.schur(0)
    cols, precs = [np.ones(n)], [0.01]
    for s_ in loci:
        cols.append(H.coding(g[s_], 0))
        precs.append(itv[0])
    X = np.stack(cols, 1)
    base = H.lml_numpy(X, y, np.array(precs), 2 * 0.7 + y @ y, n + 2)
    assert base == pytest.approx(st.log_likelihood, rel=1e-10)
    checked = 0
    for j in range(p):
        if j in set(loci.tolist()):
            assert np.isnan(dl[j, 0])
            continue
        Xj = np.column_stack([X, H.coding(g[j], 0)])
        exp = H.lml_numpy(Xj, y, np.array(precs + [itv[0]]), 2 * 0.7 + y @ y, n + 2) - base
        assert dl[j, 0] == pytest.approx(exp, rel=1e-9, abs=1e-9)
        checked += 1
    assert checked == p - len(loci)


def test_proposal_tree_known_answers(oracle):
    """DiscreteDistributionTests.{Construction,Updates} (src/tests/discrete_distribution_tests.hpp:31-200):
    node values (own weight plus the left subtree) and the total after zeroing
    and restoring SNPs; switchdate(a, b) is written as zeroing a and restoring b."""
    w = [0.1, 0.2, 0.3, 0.4, 0.5]
    full = [0.1 + 0.2 + 0.4 + 0.5, 0.2 + 0.4, 0.3, 0.4, 0.5]
    steps = [
        ([], full, 1.5),
        ([0], [0.2 + 0.4 + 0.5, 0.6, 0.3, 0.4, 0.5], 1.4),
        ([0, 4], [0.6, 0.6, 0.3, 0.4, 0.0], 0.9),
        ([0, 4, 2], [0.6, 0.6, 0.0, 0.4, 0.0], 0.6),
        ([0, 4, 2, -1], [0.7, 0.6, 0.0, 0.4, 0.0], 0.7),
        ([0, 4, 2, -1, 3, -3, 2, -4, 3, -3], [0.1 + 0.2, 0.2, 0.3, 0.0, 0.0], 0.6),
        ([0, 4, 2, -1, 3, -3, 2, -4, 3, -3, -5, -4], full, 1.5),
        ([0, 1, 2, 3, 4], [0.0] * 5, 0.0),
        ([0, 1, 2, 3, 4, -1, -2, -3, -4, -5], full, 1.5),
    ]
    for ops, values, total in steps:
        v, t, _ = oracle.dd_exercise(w, ops)
        np.testing.assert_allclose(v, values, rtol=0, atol=1e-15, err_msg=str(ops))
        assert t == pytest.approx(total, abs=1e-15), ops
    # many zero/restore rounds leave the tree where it started
    rng = np.random.default_rng(1234)
    ops = []
    for ind in rng.integers(0, 5, size=200000):
        ind = int(ind)
        ops += [ind, (ind + 2) % 5, (ind + 1) % 5, -ind - 1, -((ind + 2) % 5) - 1, -((ind + 1) % 5) - 1]
    v, t, _ = oracle.dd_exercise(w, ops)
    np.testing.assert_allclose(v, full, rtol=0, atol=1e-15)
    assert t == pytest.approx(1.5, abs=1e-15)


def test_proposal_tree_sampling(oracle):
    """DiscreteDistributionTests.{Sample,SampleManySizes,SampleSomeZeroed}
    (src/tests/discrete_distribution_tests.hpp:202-385): draw frequencies
    match the normalised weights of the SNPs that are not zeroed (1M draws per
    case, 0.002 absolute)."""
    _, _, c = oracle.dd_exercise([0.1, 0.001, 0.3, 0.099, 0.5], n_samples=1000000)
    np.testing.assert_allclose(c / 1e6, [0.1, 0.001, 0.3, 0.099, 0.5], rtol=0, atol=0.002)
    rng = np.random.default_rng(1234)
    for size in range(1, 32):
        p = rng.random(size)
        p /= p.sum()
        zero = rng.choice(size, size // 2, replace=False) if size < 16 else np.array([], dtype=int)
        _, t, c = oracle.dd_exercise(p, list(zero), seed=size, n_samples=1000000)
        q = p.copy()
        q[zero] = 0
        assert t == pytest.approx(q.sum(), rel=1e-12)
        np.testing.assert_allclose(c / 1e6, q / q.sum(), rtol=0, atol=0.002, err_msg="size %d" % size)


@pytest.mark.parametrize("types", [[0], [0, 4], [0, 1, 2, 3, 4]], ids=["A", "A_AH", "all"])
def test_missing_call_imputation_known_answers(bmg, oracle, types):
    """DataModelTests.{MissingSampling,XXUpdatesA,XXUpdatesAAH,XXUpdatesAll}
    (src/tests/data_model_tests.hpp:129-322) on plinktest (n = 5, SNP 0 has a
    missing call): the imputed value follows SNP 0's observed genotype
    frequencies (0.25, 0.25, 0.5), and after every draw the corrected
    precomputed sums equal the sums of the imputed codings."""
    z = H.golden("data_tests")
    packed, n = z["plink_bed"][3:], 5
    fam = z["plink_fam"].tobytes().decode().split()
    y = np.array([float(fam[6 * i + 5]) for i in range(n)])
    o = small_opts(bmg, n, 10, types, recode_g_to_minor_allele_count=0)
    port = oracle.Port(o, packed, y)
    counts, _, g = port.missing_step(0, n_reps=100000)
    assert g[0][3] >= 0
    np.testing.assert_allclose(counts / counts.sum(), [0.25, 0.25, 0.5], atol=0.01)
    terms = sorted({t for ty in types for t in ((0, 1) if ty == 4 else (ty,))})
    for _ in range(100):
        for snp in (0, 3):
            _, xx, g = port.missing_step(snp, n_reps=1 if snp == 0 else 0)
            assert np.all(g >= 0)
            for k, t in enumerate(terms):
                x = g[t]
                assert xx[2 * k] == pytest.approx(x.sum(), abs=1e-12)
                assert xx[2 * k + 1] == pytest.approx(x @ x - x.sum() ** 2 / n, abs=1e-12)
            if 4 in types:
                a, h = g[0], g[1]
                assert xx[-1] == pytest.approx(a @ h - a.sum() * h.sum() / n, abs=1e-10)


def test_sigma2_beta_draws_follow_their_posterior(bmg, oracle):
    """ModelTests.Sigma2BetaSampling (src/tests/model_tests.hpp:314-410):
    draws of (sigma2, beta) given the constant-only model and given the model
    with SNP 5 in A,H coding, on plinktest with nu_sigma2 = 0.  The reference's
    constants (the residual sums of squares and the posterior means) are
    checked against the closed form, and 1M draws through the oracle's random
    stream against the closed-form moments: S / sigma2 ~ chi2(n) (its mean and
    variance), and the mean and variance of each coefficient (a Student t with
    n degrees of freedom around the posterior mean, scale sigma2 A^-1)."""
    z = H.golden("data_tests")
    packed, n = z["plink_bed"][3:], 5
    fam = z["plink_fam"].tobytes().decode().split()
    y = np.array([float(fam[6 * i + 5]) for i in range(n)])
    o = small_opts(bmg, n, 10, [0, 4], e_qg=2, var_qg=4, nu_sigma2=0, s2_sigma2=1, mu_alpha=1,
                   inv_tau2_e_const_val=0, recode_g_to_minor_allele_count=0)
    port = oracle.Port(o, packed, y)
    inv = 1.0 / (1.0 * 1.0 * (4.0 * 1.0 / (4.0 - 2.0)))
    g = H.decode(packed, n, 10)
    cases = [
        ([], np.ones((n, 1)), np.array([0.0]), 0.0680, [0.32]),
        ([5], np.column_stack([np.ones(n), H.coding(g[5], 0), H.coding(g[5], 1)]), np.array([0.0, inv, inv]),
         0.02988235294117647101, [None, -0.11999999999999999556, -0.03529411764705892018]),
    ]
    N = 1000000
    for snps, X, prec, syy_ref, means_ref in cases:
        A = X.T @ X + np.diag(prec)
        Ainv = np.linalg.inv(A)
        mu = Ainv @ X.T @ y
        S = y @ y - (X.T @ y) @ mu
        assert S == pytest.approx(syy_ref, rel=1e-9)
        for m_ref, m in zip(means_ref, mu):
            if m_ref is not None:
                assert m == pytest.approx(m_ref, rel=1e-9, abs=1e-12)
        s2, beta = port.sample_beta_sigma2(snps, [1] * len(snps), [[inv, inv]] * len(snps), N, seed=1234)
        q = S / s2
        assert q.mean() == pytest.approx(n, abs=0.02)
        assert q.var() == pytest.approx(2 * n, abs=0.15)
        es2 = S / (n - 2)
        for j in range(len(mu)):
            sd = np.sqrt(es2 * Ainv[j, j])
            assert beta[:, j].mean() == pytest.approx(mu[j], abs=6 * sd / np.sqrt(N))
            assert beta[:, j].var() == pytest.approx(es2 * Ainv[j, j], rel=0.02)


def test_model_prior_changes_known_answer(bmg, oracle):
    """PriorTests.SimpleAddRemove (src/tests/prior_tests.hpp:31-125): with
    e_qg = 3, var_qg = 9 and types A, AH, each change on add, remove and type
    switch equals the difference of the log model priors (1e-6 there; 1e-12
    here)."""
    z = H.golden("data_tests")
    packed, n = z["plink_bed"][3:], 5
    fam = z["plink_fam"].tobytes().decode().split()
    y = np.array([float(fam[6 * i + 5]) for i in range(n)])
    o = small_opts(bmg, n, 10, [0, 4], e_qg=3, var_qg=9, nu_sigma2=1, s2_sigma2=1, mu_alpha=1,
                   inv_tau2_e_const_val=0)
    for t in range(4):
        o.nu_tau2[t], o.s2_tau2[t] = 3, 1
    port = oracle.Port(o, packed, y)
    A, AH = 0, 4
    lm = lambda ns: port.prior_terms(ns, 0, A)[0]
    for ns, ns_new, nl, t in [([0, 0, 0, 0, 0], [1, 0, 0, 0, 0], 0, A), ([2, 0, 0, 0, 3], [3, 0, 0, 0, 3], 5, A),
                              ([0, 0, 0, 0, 0], [0, 0, 0, 0, 1], 0, AH), ([3, 0, 0, 0, 2], [3, 0, 0, 0, 3], 5, AH)]:
        assert port.prior_terms(ns, nl, t)[1] == pytest.approx(lm(ns_new) - lm(ns), abs=1e-12)
        assert port.prior_terms(ns_new, nl + 1, t)[2] == pytest.approx(lm(ns) - lm(ns_new), abs=1e-12)
    same = [3, 0, 0, 0, 3]
    assert port.prior_terms(same, 6, AH, AH)[3] == pytest.approx(0.0, abs=1e-12)
    ns, ns_new = [3, 0, 0, 0, 2], [2, 0, 0, 0, 3]
    assert port.prior_terms(ns, 5, AH, A)[3] == pytest.approx(lm(ns_new) - lm(ns), abs=1e-12)
    assert port.prior_terms(ns_new, 5, A, AH)[3] == pytest.approx(lm(ns) - lm(ns_new), abs=1e-12)
