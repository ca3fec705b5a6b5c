"""GPU parity against the reference's traces for the options the main parity
file does not cover: the flat proposal with the beta trace and raw
genotypes, a model past the 128 columns kept in shared memory, individual
tau2 over five effect types, delayed rejection (the second stage over all
sub-models of a rejected multi-SNP or state-change move: one and two effect
types, and the reference example's delay_rejection = 10 with covariates),
missing genotype calls (imputed at every RB step and with every new term, and
Gibbs-updated in the model: src/data_model.cpp:30-167, src/sampler.cpp:264-453)
and the command-line entry end to end."""
import numpy as np
import pytest

import helpers as H
from test_gpu_parity import RTOL, run_gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["small_flat", "example_flat", "example_large", "example_types_indiv",
                                  "small_dr", "example_dr", "small_types_dr",
                                  "small_types_missing", "example_missing", "small_types_dr_missing"])
def test_gpu_matches_reference_more_options(bmg, tmp_path, name):
    """A flat proposal with the beta trace and raw genotypes (small_flat,
    example_flat), a model that grows past the 128 columns the move kernel
    keeps in shared memory (example_large), individual tau2 draws over four
    terms in the scan (example_types_indiv), delayed rejection (small_dr,
    example_dr, small_types_dr: src/sampler.cpp:882-1049,
    src/sampler.hpp:929-1098, 1547-1618) and missing calls (5 % of the calls
    with A and AH, 2 % with covariates and individual tau2, and missing calls
    with delayed rejection), against the reference's traces."""
    z = H.golden("ref_" + name)
    ini = H.materialize(z, tmp_path)
    opt = bmg.options_from_ini(ini)
    packed, y, e = bmg.read_plink(opt)
    ctx, col = run_gpu(bmg, opt, packed, y, e, opt.do_n_iter)
    for c in range(opt.n_chains):
        ref = H.ref_chain(z, c)
        got = col.chain(c)
        H.compare(ref, got, rtol=RTOL, label="%s chain %d" % (name, c))
        if "c%d_beta" % c in z.files:
            np.testing.assert_allclose(got["beta"], z["c%d_beta" % c], rtol=1e-7, atol=1e-10)
        np.testing.assert_allclose(ctx.rao(c)[0], ref["rao"], rtol=RTOL, atol=1e-12)


def test_cli_writes_the_reference_files(bmg, tmp_path):
    """bmagwa-gb300 INIFILE end to end: the trace files equal the reference's."""
    import os
    import subprocess
    z = H.golden("ref_small")
    ini = H.materialize(z, tmp_path)
    cli = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bmagwa_gb300", "_build",
                       "bmagwa-gb300")
    r = subprocess.run([cli, ini], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    import oracle.port as op
    for c in range(2):
        out = op.read_ref_outputs(str(tmp_path / "out" / "chain"), c, 7)
        H.compare(H.ref_chain(z, c), out, rtol=RTOL, label="cli chain %d" % c)
