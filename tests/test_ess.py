"""The inclusion-indicator ESS estimator on series with a known answer."""
import numpy as np
import pytest

from bmagwa_gb300 import ess


def _markov01(T, stay, seed):
    """Symmetric two-state chain: P(stay) = stay; lag-k autocorrelation
    (2 stay - 1)^k, so tau = (1 + r) / (1 - r) with r = 2 stay - 1."""
    rng = np.random.default_rng(seed)
    x = np.empty(T)
    x[0] = 0
    u = rng.random(T)
    for t in range(1, T):
        x[t] = x[t - 1] if u[t] < stay else 1 - x[t - 1]
    return x


@pytest.mark.parametrize("stay", [0.5, 0.8, 0.95])
def test_ess_matches_two_state_chain(stay):
    T = 200000
    x = _markov01(T, stay, 7)
    r = 2 * stay - 1
    tau = (1 + r) / (1 - r)
    assert ess.ess_geyer(x) == pytest.approx(T / tau, rel=0.1)


def test_constant_series_has_no_ess():
    assert np.isnan(ess.ess_geyer(np.ones(50)))


def test_indicator_matrix_and_filter():
    # three samples: {5, 9}, {9}, {} ; then repeat
    ms = np.array([2, 1, 0] * 20)
    loci = np.array([5, 9, 9] * 20)
    G, snps = ess.indicator_matrix(ms, loci)
    assert list(snps) == [5, 9]
    assert G[:3].tolist() == [[1, 1], [0, 1], [0, 0]]
    s, e = ess.inclusion_ess(ms, loci)
    assert set(s.tolist()) == {5, 9} and np.all(e > 0)
    out = ess.summarize([(ms, loci)], seconds=2.0)
    assert out["snps"] == 2 and out["per_s"] > 0
