"""Host-side logic of libbmg on the CPU: the C ABI's exported symbols, the INI
option rules (src/options.hpp:138-321, src/inih/ini.c:57-130) and the PLINK
readers (src/data.cpp:141-273).  Nothing here launches a kernel."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest
import torch

import bmagwa_gb300 as bg
from bmagwa_gb300 import nvbuild
from bmagwa_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "bmg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bmg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    names = _declared_symbols()
    assert "bmg_run" in names and "bmg_precompute_noalloc" in names
    L = C.CDLL(nvbuild.LIB)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings():
    L = bg.lib()
    L.bmg_status_string.restype = C.c_char_p
    seen = set()
    for code in range(0, 9):
        s = L.bmg_status_string(code)
        assert s and s.decode()
        seen.add(s)
    assert len(seen) == 9


def _ini(tmp_path, **repl):
    path = synth.write_ini(str(tmp_path / "run.ini"), "t", str(tmp_path / "data"), str(tmp_path),
                           n=100, p=50, chains=2, types="A", n_rao=10, iters=100)
    txt = open(path).read()
    for k, v in repl.items():
        if v is None:
            txt = re.sub(r"(?m)^%s\s*=.*\n" % k, "", txt)
        else:
            txt = re.sub(r"(?m)^%s\s*=.*$" % k, "%s = %s" % (k, v), txt)
    open(path, "w").write(txt)
    return path


def test_options_from_synthetic_ini(tmp_path):
    o = bg.options_from_ini(_ini(tmp_path))
    assert (o.n, o.m_g, o.m_e, o.n_chains) == (100, 50, 0, 2)
    assert (o.do_n_iter, o.n_rao, o.thin) == (100, 10, 10)
    assert o.n_types == 1 and o.types[0] == 0
    assert list(o.seeds[:2]) == [1, 1001]
    assert o.p_move_size == pytest.approx(0.2)


def test_types_are_sorted_and_each_needs_its_prior(tmp_path):
    o = bg.options_from_ini(_ini(tmp_path, types="H, A"))
    assert o.n_types == 2 and [o.types[i] for i in range(2)] == [0, 1]
    # the template sets priors for A and H only
    with pytest.raises(bg.BmgError, match=re.escape("Cannot leave option empty: prior.nu_tau2_R")):
        bg.options_from_ini(_ini(tmp_path, types="AH, R"))


@pytest.mark.parametrize("key,value,msg", [
    ("n", None, "Cannot leave option empty: sizes.n"),
    ("n", "0", "Positive integer required"),
    ("n", "12x", "Invalid conversion"),
    ("thin", "3", "n_rao should be a multiple of thin"),
    ("seeds", "1", "Number of seeds must equal n_threads"),
    ("seeds", "5, 5", "Seeds are not unique"),
    ("types", "A, Q", "Unknown model type"),
    ("type", "XYZ", "unknown sampler type"),
    ("p_move_size", "1.5", "p_move_size must be <= 1"),
    ("adaptation", "2", "Boolean value required"),
    ("R2mode_sigma2", "1.5", "Value in 0..1 required"),
    ("nu_sigma2", "-1", "Positive value required for prior.nu_sigma2"),
])
def test_option_errors(tmp_path, key, value, msg):
    with pytest.raises(bg.BmgError, match=re.escape(msg)):
        bg.options_from_ini(_ini(tmp_path, **{key: value}))


def test_ini_grammar(tmp_path):
    """Comments, ':' separators, case-insensitive keys, inline ';' comments
    after whitespace, continuation lines and later-key-wins."""
    path = _ini(tmp_path)
    txt = open(path).read()
    txt = txt.replace("[sizes]\nn = 100", "[SIZES]\n# a comment\nN : 7 ; inline comment\nn = 100")
    txt = txt.replace("do_n_iter = 100", "do_n_iter =\n   250")
    open(path, "w").write(txt)
    o = bg.options_from_ini(path)
    assert o.n == 100 and o.do_n_iter == 250


def test_ini_syntax_error_and_missing_file(tmp_path):
    path = _ini(tmp_path)
    open(path, "a").write("\n[broken\n")
    with pytest.raises(bg.BmgError, match="Cannot load/parse"):
        bg.options_from_ini(path)
    with pytest.raises(bg.BmgError, match="Cannot load/parse"):
        bg.options_from_ini(str(tmp_path / "absent.ini"))


def _plink(tmp_path, n=37, p=9, seed=3):
    rng = np.random.default_rng(seed)
    g = rng.integers(0, 3, size=(p, n))
    y = rng.normal(size=n)
    prefix = str(tmp_path / "data")
    synth.write_plink(prefix, synth.pack(torch.as_tensor(g)), y)
    ini = synth.write_ini(str(tmp_path / "run.ini"), "t", prefix, str(tmp_path), n=n, p=p, chains=1,
                          types="A", n_rao=10, iters=10)
    return ini, prefix, g, y


def test_read_plink_roundtrip(tmp_path):
    ini, prefix, g, y = _plink(tmp_path)
    o = bg.options_from_ini(ini)
    packed, y2, e = bg.read_plink(o)
    assert e is None
    np.testing.assert_array_equal(y2, np.array([float("%.17g" % v) for v in y]))
    stride = (g.shape[1] + 3) // 4
    codes = np.unpackbits(packed.reshape(-1, stride)[:, :, None], axis=2, bitorder="little")
    codes = (codes[:, :, 0::2] + 2 * codes[:, :, 1::2]).reshape(g.shape[0], -1)[:, :g.shape[1]]
    # PLINK codes: 0 hom-ref, 2 het, 3 hom-alt, 1 missing
    dec = np.select([codes == 0, codes == 2, codes == 3], [0, 1, 2], -1)
    np.testing.assert_array_equal(dec, g)


def test_read_plink_errors(tmp_path):
    ini, prefix, g, y = _plink(tmp_path)
    o = bg.options_from_ini(ini)
    bed = open(prefix + ".bed", "rb").read()
    open(prefix + ".bed", "wb").write(b"\x6c\x1b\x00" + bed[3:])
    with pytest.raises(bg.BmgError, match="snp-major"):
        bg.read_plink(o)
    open(prefix + ".bed", "wb").write(b"\x00" + bed[1:])
    with pytest.raises(bg.BmgError, match="magic number"):
        bg.read_plink(o)
    open(prefix + ".bed", "wb").write(bed[:-1])
    with pytest.raises(bg.BmgError, match="Reading the BED file failed"):
        bg.read_plink(o)
    open(prefix + ".bed", "wb").write(bed)
    fam = open(prefix + ".fam").read().splitlines()
    open(prefix + ".fam", "w").write("\n".join(fam[:-1]) + "\n")
    with pytest.raises(bg.BmgError, match="FAM file size does not match given n"):
        bg.read_plink(o)


def test_alternate_phenotype_and_covariates(tmp_path):
    ini, prefix, g, y = _plink(tmp_path, n=11, p=4)
    fam = [l.split() for l in open(prefix + ".fam").read().splitlines()]
    rng = np.random.default_rng(9)
    yalt = rng.normal(size=len(fam))
    ecov = rng.normal(size=(len(fam), 2))
    order = rng.permutation(len(fam))
    with open(prefix + ".y", "w") as f:
        for i in order:
            f.write("%s %s %.17g\n" % (fam[i][0], fam[i][1], yalt[i]))
        f.write("nobody nobody 1.0\n")
    def write_e(nan_first):
        with open(prefix + ".e", "w") as f:
            if nan_first:
                f.write("%s %s nan 1.0\n" % (fam[0][0], fam[0][1]))
            for i in order:
                f.write("%s %s %.17g %.17g\n" % (fam[i][0], fam[i][1], ecov[i, 0], ecov[i, 1]))
            f.write("%s %s nan 1.0\n" % (fam[0][0], fam[0][1]))

    write_e(False)
    txt = open(ini).read()
    txt = txt.replace("file_g = %s.bed" % prefix, "file_g = %s.bed\nfile_y = %s.y\nfile_e = %s.e" % (prefix, prefix, prefix))
    txt = txt.replace("m_e = 0", "m_e = 2")
    open(ini, "w").write(txt)
    o = bg.options_from_ini(ini)
    _, y2, e = bg.read_plink(o)
    np.testing.assert_array_equal(y2, yalt)
    np.testing.assert_array_equal(e.reshape(2, -1).T, ecov)
    # a literal "nan" fails the stream extraction, which ends the file there
    # (src/data.cpp:208-216), so rows after it are never read
    write_e(True)
    with pytest.raises(bg.BmgError, match="Covariate file does not contain all covariates"):
        bg.read_plink(o)
    write_e(False)
    # drop one row of the alternate phenotypes
    lines = open(prefix + ".y").read().splitlines()
    open(prefix + ".y", "w").write("\n".join(lines[1:]) + "\n")
    with pytest.raises(bg.BmgError, match="Alternate phenotype file does not contain all phenotypes"):
        bg.read_plink(o)


def test_create_rejects_unsupported_options_before_touching_the_device(tmp_path):
    """Option checks of bmg_create run before any CUDA call, so they hold on
    a host without a GPU too."""
    o = bg.options_from_ini(_ini(tmp_path))
    h = C.c_void_p()
    L = bg.lib()
    for field, value, status in [("max_SNP_neighborhood_size", 129, "BMG_EINVAL"),
                                 ("delay_rejection", 17, "BMG_EUNSUPPORTED"),
                                 ("sampler_type", 1, "BMG_EUNSUPPORTED")]:
        old = getattr(o, field)
        setattr(o, field, value)
        rc = L.bmg_create(C.byref(o), C.byref(h))
        L.bmg_status_string.restype = C.c_char_p
        assert L.bmg_status_string(rc).decode() == status, field
        assert h.value is None
        # the message of a failed create stays readable without a context
        assert len(L.bmg_last_error(None)) > 10, field
        with pytest.raises(bg.BmgError, match=status):
            bg.Context(o)
        setattr(o, field, old)


def test_options_struct_matches_the_library():
    L = bg.lib()
    L.bmg_options_size.restype = C.c_size_t
    from bmagwa_gb300 import abi
    assert L.bmg_options_size() == C.sizeof(abi.Options)
    o = bg.default_options()
    assert o.learned_topk == 1024 and o.learned_mix == pytest.approx(0.3)


def test_library_free_defaults_equal_the_library_defaults():
    """abi.default_options (used where only the oracle runs) fills every
    field as bmg_options_default does."""
    from bmagwa_gb300 import abi
    a, b = abi.default_options(), bg.default_options()
    assert C.string_at(C.addressof(a), C.sizeof(a)) == C.string_at(C.addressof(b), C.sizeof(b))


def _option_cases():
    with open(os.path.join(os.path.dirname(__file__), "golden", "options_ref.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("case", _option_cases(), ids=lambda c: c["name"])
def test_options_match_the_reference_parser(tmp_path, capfd, case):
    """bmg_options_from_ini against the reference's own parser
    (src/options.hpp:138-321, run over the same INI text by
    tests/golden/make_golden.py): every field, the error message, and the
    default-value warnings in the order printed."""
    path = tmp_path / "opt.ini"
    path.write_text(case["ini"])
    ref = case["fields"]
    capfd.readouterr()
    if "error" in ref:
        with pytest.raises(bg.BmgError) as ei:
            bg.options_from_ini(str(path), quiet=False)
        assert str(ei.value).split(": ", 1)[1] == ref["error"]
        return
    o = bg.options_from_ini(str(path), quiet=False)
    out = capfd.readouterr().out
    warnings = [ln for ln in out.splitlines() if ln.startswith("Warning")]
    assert warnings == case["warnings"]
    for k in ("file_fam", "file_g", "file_e", "file_y", "basename"):
        assert getattr(o, k).decode() == ref[k], k
    ints = ("n", "m_g", "m_e", "recode_g_to_minor_allele_count", "sampler_type", "do_n_iter", "n_rao",
            "n_rao_burnin", "thin", "n_sample_tau2_and_missing", "max_move_size", "max_SNP_neighborhood_size",
            "adapt_p_move_size", "adaptation", "flat_proposal_dist", "save_beta", "verbosity", "delay_rejection",
            "n_chains", "use_individual_tau2")
    for k in ints:
        assert int(getattr(o, k)) == int(ref[k]), k
    reals = ("p_move_size", "p_move_size_nbs", "p_move_size_nbc", "p_move_size_acpt_goal", "e_qg", "var_qg",
             "nu_sigma2", "s2_sigma2", "R2mode_sigma2", "mu_alpha", "inv_tau2_e_const_val", "inv_tau2_e_val")
    for k in reals:
        assert getattr(o, k) == float(ref[k]), k
    types = [int(t) for t in ref["types"].split(",")]
    assert [o.types[i] for i in range(o.n_types)] == types
    assert list(o.seeds[:o.n_chains]) == [int(s) for s in ref["seeds"].split(",")]
    for t in range(5):
        assert o.types_prior[t] == float(ref["types_prior.%d" % t]), t
    terms = {t for ty in types for t in ((0, 1) if ty == 4 else (ty,))}
    for t in terms:
        for k in ("nu_tau2", "s2_tau2", "eh_tau2"):
            assert getattr(o, k)[t] == float(ref["%s.%d" % (k, t)]), (k, t)


def _reader_cases():
    with open(os.path.join(os.path.dirname(__file__), "golden", "readers_ref.json")) as f:
        return json.load(f)


def _materialize_reader_case(tmp_path, case):
    import base64
    for fn, v in case["files"].items():
        data = base64.b64decode(v) if fn.endswith(".bed") else v.encode()
        (tmp_path / fn).write_bytes(data)
    ini = tmp_path / "r.ini"
    ini.write_text(case["ini"].replace("{DIR}", str(tmp_path)))
    return str(ini)


@pytest.mark.parametrize("case", _reader_cases(), ids=lambda c: c["name"])
def test_readers_match_the_reference_data_class(tmp_path, oracle, case):
    """bmg_read_plink against the reference's Data class (src/data.cpp:141-273,
    run on the same files by tests/golden/make_golden.py): the phenotypes of
    the .fam or the alternate .y file, the covariates of the .e file, and the
    error message of each malformed input; the oracle's summary statistics
    (src/data.hpp:45-72) on the data read."""
    o = bg.options_from_ini(_materialize_reader_case(tmp_path, case))
    ref = case["result"]
    if "error" in ref:
        with pytest.raises(bg.BmgError) as ei:
            bg.read_plink(o)
        assert str(ei.value).split(": ", 1)[1] == ref["error"]
        return
    packed, y, e = bg.read_plink(o)
    n = int(o.n)
    assert [float(ref["y.%d" % i]) for i in range(n)] == list(y)
    if o.m_e:
        e = np.asarray(e).reshape(o.m_e, n)
        for j in range(o.m_e):
            assert [float(ref["e.%d.%d" % (j, i)]) for i in range(n)] == list(e[j]), j
    port = oracle.Port(o, packed, y, e if o.m_e else None)
    var_x, mean_x, var_y, yy = port.data_stats()
    assert (var_x, mean_x, var_y, yy) == tuple(float(ref[k]) for k in ("var_x", "mean_x", "var_y", "yy"))


def test_fam_with_more_rows_than_n_is_an_error(tmp_path):
    """A .fam with n + 1 rows: the reference writes past its phenotype vector
    before checking the count (src/data.cpp:158-166); the product reports the
    count error the reference's check names."""
    case = _reader_cases()[0]
    fam = case["files"]["d.fam"]
    case = dict(case, files=dict(case["files"], **{"d.fam": fam + "F9 I99 0 0 1 0.5\n"}))
    o = bg.options_from_ini(_materialize_reader_case(tmp_path, case))
    with pytest.raises(bg.BmgError, match="FAM file size does not match given n"):
        bg.read_plink(o)
