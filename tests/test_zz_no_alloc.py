"""bmg_precompute_noalloc: the entry point for callers that cannot allocate
device memory (a foreign memory pool, a stream under capture).  It must give
the oracle's precomputed per-SNP sums (PrecomputedSNPCovariances::precompute,
src/precomputed_snp_covariances.hpp:95-131, missing calls counted as 0 as
they are before any imputation), and what a context's bmg_get_precomputed
gives, call after call, from buffers the caller owns, with its working memory
inside the library.  The file sorts last so that a run stopping at the first
failure has run every other test first."""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _noalloc(bmg, packed, n, p, recode, types, calls=2):
    """Two calls in a row on the same caller buffers; returns the outputs."""
    import torch
    d_packed = torch.from_numpy(np.ascontiguousarray(packed)).cuda()
    d_flag = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    out = []
    d_out = None
    for _ in range(calls):
        if d_out is None:
            d_out = torch.full((p * 16,), float("nan"), dtype=torch.float64, device="cuda")
        d_out.fill_(float("nan"))
        d_flag.fill_(7)
        torch.cuda.synchronize()
        off = bmg.precompute_noalloc(d_packed.data_ptr(), n, p, recode, types, d_out.data_ptr(),
                                     d_flag.data_ptr())
        torch.cuda.synchronize()
        out.append((off, d_out[:p * off].cpu().numpy().reshape(p, off).copy(), int(d_flag.item())))
    return out


@pytest.mark.parametrize("fixture,types", [
    ("ref_example", None), ("ref_example", [0, 4]), ("ref_example", [0, 1, 2, 3, 4]),
    ("ref_small_types_missing", None), ("ref_example_missing", None),
], ids=["example_A", "example_A_AH", "example_all", "small_missing_A_AH", "example_missing_A"])
def test_precompute_noalloc_matches_oracle(bmg, oracle, tmp_path, fixture, types):
    z = H.golden(fixture)
    ini = H.materialize(z, tmp_path)
    opt = bmg.options_from_ini(ini)
    if types is not None:
        opt.n_types = len(types)
        for i, t in enumerate(types):
            opt.types[i] = t
        for t in range(4):
            opt.nu_tau2[t], opt.s2_tau2[t] = 5, 0.05
    types = [int(opt.types[i]) for i in range(opt.n_types)]
    packed, y, e = bmg.read_plink(opt)
    n, p = int(opt.n), int(opt.m_g)
    ref = oracle.Port(opt, packed, y, e).precomputed()
    has_missing = bool((H.decode(packed, n, p) < 0).any())
    for call, (off, got, flag) in enumerate(_noalloc(bmg, packed, n, p, opt.recode_g_to_minor_allele_count,
                                                     types)):
        assert off == ref.shape[1]
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12, err_msg="call %d" % call)
        assert flag == int(has_missing), "call %d" % call
    if not has_missing:
        # and what a context computes for the same data
        ctx = bmg.Context(opt)
        ctx.load_bed(packed)
        ctx.set_phenotypes(y)
        ctx.set_covariates(e)
        ctx.precompute()
        np.testing.assert_allclose(ctx.precomputed(), ref, rtol=1e-12, atol=1e-12)
        ctx.close()


def test_precompute_noalloc_rejects_oversize(bmg):
    import torch
    d = torch.zeros(16, dtype=torch.uint8, device="cuda")
    out = torch.zeros(16, dtype=torch.float64, device="cuda")
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(bmg.BmgError):
        bmg.precompute_noalloc(d.data_ptr(), 4, (1 << 20) + 1, 0, [0], out.data_ptr(), flag.data_ptr())
    assert "2^20" in bmg.lib().bmg_last_error(None).decode()
    with pytest.raises(bmg.BmgError):
        bmg.precompute_noalloc(d.data_ptr(), 1 << 31, 4, 0, [0], out.data_ptr(), flag.data_ptr())
    assert "2^31" in bmg.lib().bmg_last_error(None).decode()
