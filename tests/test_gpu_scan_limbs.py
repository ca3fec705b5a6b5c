"""How many base-256 residual limbs the RB scan needs: the per-SNP log
posterior odds against the FP64 oracle (RaoBlackwellizer::p_raoblackwell,
src/sampler.cpp:32-261, with the same fitted values and sigma2) for four,
five and six limbs on the `scan` workload's data at p = 100,000.  Six (the
default) stay far inside the 1e-9 relative tolerance the parity tests use;
five come within a factor of a few of it (trajectory tests at 1e-9 then fail
on p_rao), four exceed it.  The errors are printed per limb count."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_residual_limbs_against_the_fp64_oracle(bmg, oracle):
    from bmagwa_gb300 import workloads
    wl = dict(workloads.WORKLOADS["scan"], p=100000, chains=2)
    packed, y = workloads.make_data(wl, 1, "cuda")
    rng = np.random.default_rng(5)
    worst = {}
    for a, noise, s2 in [(0.35, 0.05, 0.6), (0.8, 0.3, 0.2), (0.0, 0.0, 1.0)]:
        yhat = a * y + noise * rng.normal(size=y.size)
        port = oracle.Port(workloads.options(wl, 1, 1), packed, y)
        ref = port.scan_yhat_logodds(yhat, s2, 0)
        for L in (4, 5, 6):
            o = workloads.options(wl, 1, 1)
            o.scan_limbs = L
            ctx = bmg.Context(o)
            ctx.load_bed(packed)
            ctx.set_phenotypes(y)
            ctx.set_covariates(None)
            ctx.precompute()
            _, lo = ctx.scan_yhat(yhat, s2)
            ctx.close()
            rel = float((np.abs(lo[0] - ref) / np.maximum(np.abs(ref), 1.0)).max())
            worst[L] = max(worst.get(L, 0.0), rel)
    print("largest relative error of the log odds per limb count:", worst)
    assert worst[6] <= 1e-10
    assert worst[4] > 1e-9
