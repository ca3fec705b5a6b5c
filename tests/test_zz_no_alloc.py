"""bmg_precompute_noalloc: the entry point for callers that cannot allocate
device memory (a foreign memory pool, a stream under capture).  It must give
what a context's bmg_get_precomputed gives, call after call, from buffers the
caller owns, with its working memory inside the library."""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("types", [[0], [0, 4], [0, 1, 2, 3, 4]])
def test_precompute_noalloc_matches_context(bmg, tmp_path, types):
    import torch
    z = H.golden("ref_example")
    ini = H.materialize(z, tmp_path)
    opt = bmg.options_from_ini(ini)
    opt.n_types = len(types)
    for i, t in enumerate(types):
        opt.types[i] = t
    for t in range(4):
        opt.nu_tau2[t], opt.s2_tau2[t] = 5, 0.05
    packed, y, e = bmg.read_plink(opt)
    ctx = bmg.Context(opt)
    ctx.load_bed(packed)
    ctx.set_phenotypes(y)
    ctx.set_covariates(e)
    ctx.precompute()
    ref = ctx.precomputed()
    ctx.close()
    n, p = int(opt.n), int(opt.m_g)
    d_packed = torch.from_numpy(packed.copy()).cuda()
    d_out = torch.full((ref.size,), float("nan"), dtype=torch.float64, device="cuda")
    d_flag = torch.ones(1, dtype=torch.int32, device="cuda")
    for call in range(2):
        d_out.fill_(float("nan"))
        torch.cuda.synchronize()
        off = bmg.precompute_noalloc(d_packed.data_ptr(), n, p, opt.recode_g_to_minor_allele_count,
                                     types, d_out.data_ptr(), d_flag.data_ptr())
        torch.cuda.synchronize()
        assert off == ref.shape[1]
        got = d_out.cpu().numpy().reshape(p, off)
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12, err_msg="call %d" % call)
        assert int(d_flag.item()) == 0


def test_precompute_noalloc_rejects_oversize(bmg):
    import torch
    d = torch.zeros(16, dtype=torch.uint8, device="cuda")
    out = torch.zeros(16, dtype=torch.float64, device="cuda")
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")
    with pytest.raises(bmg.BmgError):
        bmg.precompute_noalloc(d.data_ptr(), 4, (1 << 20) + 1, 0, [0], out.data_ptr(), flag.data_ptr())
