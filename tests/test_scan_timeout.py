"""The failure path of the tensor-core scan's bounded waits.

Every mbarrier wait of the scan gives up after a bounded number of polls;
then the kernel records BMG_DERR_TIMEOUT, each role drains its own TMA loads
and MMAs (those drain waits keep the full bound), tensor memory is freed,
and the host call returns BMG_ETIMEOUT with the context's CUDA state intact.
Here the main-loop bound is cut to one poll (BMG_WAIT_LIMIT=1 at context
creation), so the epilogue's wait for the first tile's accumulator -- several
hundred MMA stages at n = 32,768 -- runs out on every launch.  No fault is
involved: the waits end, the copies land and the kernel returns."""
import numpy as np
import pytest

import helpers as H
from test_gpu_parity import RTOL

pytestmark = pytest.mark.gpu


def test_scan_wait_that_runs_out_returns_timeout(bmg, oracle, tmp_path, monkeypatch):
    from bmagwa_gb300 import synth, workloads
    n, p = 32768, 2048
    wl = dict(workloads.WORKLOADS["plain"], n=n, p=p, chains=2, n_rao=1)
    counts, _ = synth.genotypes(n, p, 0, 21, device="cuda")
    y, _, _ = synth.phenotype(counts, 10, 0.3, 0, 21, device="cuda")
    packed = synth.pack(counts).cpu().numpy().reshape(-1)
    del counts

    monkeypatch.setenv("BMG_WAIT_LIMIT", "1")
    monkeypatch.setenv("BMG_SCAN_VARIANT", "0")
    opt = workloads.options(wl, 9, 5)
    opt.scan_impl = 0
    ctx = bmg.Context(opt)
    ctx.load_bed(packed)
    ctx.set_phenotypes(y)
    ctx.set_covariates(None)
    ctx.precompute()
    with pytest.raises(bmg.BmgError) as err:
        ctx.scan()
    assert err.value.status == 5, str(err.value)  # BMG_ETIMEOUT
    assert "bounded device wait" in str(err.value)
    ctx.close()

    # the device is usable afterwards: a fresh context with the default bound
    # allocates tensor memory on every SM again and runs chains equal to the
    # oracle's
    monkeypatch.delenv("BMG_WAIT_LIMIT")
    monkeypatch.delenv("BMG_SCAN_VARIANT")
    opt = workloads.options(wl, 9, 5)
    opt.scan_impl = 0
    ctx = bmg.Context(opt)
    ctx.load_bed(packed)
    ctx.set_phenotypes(y)
    ctx.set_covariates(None)
    ctx.precompute()
    col = ctx.run(5)
    port = oracle.Port(workloads.options(wl, 9, 5), packed, y)
    colp = port.run(5)
    for c in range(2):
        H.compare(colp.chain(c), col.chain(c), rtol=RTOL, label="chain %d" % c)
        np.testing.assert_allclose(ctx.rao(c)[0], port.rao(c)[0], rtol=RTOL, atol=1e-12)
    ctx.close()
