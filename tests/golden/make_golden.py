"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs only where the reference tree and its oracle build (oracle/_ref) exist:

  1. known-answer vectors the reference's own tests hold, read as text from
     src/tests/data_tests.hpp (genotype matrices and phenotypes of the two test
     PLINK files), with the PLINK files themselves as byte arrays;
  2. traces of the compiled reference (oracle/_ref/bmagwa_ref, the reference
     sources built against oracle/shim) on small runs derived from the
     reference's test configurations and its example dataset, with every
     input file stored in the fixture.

Usage:  python tests/golden/make_golden.py [REFERENCE_DIR [CASE ...]]
(all cases when none is named)
"""
import base64
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle.port import reference_dir  # noqa: E402

# the reference tree: the first argument, else $BMAGWA_REFERENCE, else the
# oracle recipe's default location
REF = sys.argv[1] if len(sys.argv) > 1 else reference_dir()
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "bmagwa_ref")
REF_PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_probe")

TRACE_FILES = {
    "jumpdistance": np.uint8, "move_type": np.uint8, "move_size": np.uint8,
    "modelsize": np.uint32, "loci": np.uint32, "log_likelihood": np.float64,
    "log_prior": np.float64, "sigma2": np.float64, "alpha": np.float64, "pve": np.float64,
    "rao": np.float64, "types": np.uint8, "rao_types": np.float64, "beta": np.float64,
}


def parse_matrix(text, name):
    """Values of `const char name[..][..] = {{...},...};` in a C++ test file."""
    m = re.search(r"%s\[(\d+)\]\[(\d+)\]\s*=\s*\{(.*?)\};" % name, text, re.S)
    rows, cols = int(m.group(1)), int(m.group(2))
    vals = [int(v) for v in re.findall(r"-?\d+", m.group(3))]
    return np.array(vals, dtype=np.int8).reshape(rows, cols)


def known_answers():
    text = open(os.path.join(REF, "src/tests/data_tests.hpp")).read()
    first, second = text.split("LoadAndHandlePlinkDataWithMissing")
    g7 = parse_matrix(first, "genotypes")
    ym = re.search(r"const double y\[30\]\s*=\s*\{(.*?)\};", first, re.S)
    y30 = np.array([float(v) for v in ym.group(1).replace("\n", " ").split(",")])
    g10 = parse_matrix(second, "genotypes")
    tdir = os.path.join(REF, "src/tests/testdata")
    rd = lambda f: np.frombuffer(open(os.path.join(tdir, f), "rb").read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "data_tests.npz"),
                        small_bed=rd("small_modelspace.bed"), small_fam=rd("small_modelspace.fam"),
                        small_genotypes=g7, small_y=y30,
                        plink_bed=rd("plinktest.bed"), plink_fam=rd("plinktest.fam"),
                        plink_genotypes=g10)


INI = """[datafiles]
file_fam = {{DIR}}/data.fam
file_g = {{DIR}}/data.bed
{efile}{yfile}recode_g_to_minor_allele_count = {recode}
[sizes]
n = {n}
m_g = {p}
m_e = {m_e}
[sampler]
type = PMV
do_n_iter = {iters}
n_rao = {n_rao}
n_rao_burnin = {burnin}
adaptation = {adaptation}
verbosity = {verbosity}
thin = {thin}
n_sample_tau2_and_missing = {nst}
delay_rejection = {dr}
p_move_size = 0.2
p_move_size_nbc = 0.25
p_move_size_nbs = 0.7
max_SNP_neighborhood_size = {nbh}
adapt_p_move_size = {adapt_ms}
p_move_size_acpt_goal = {acpt}
max_move_size = {maxms}
flat_proposal_dist = {flat}
save_beta = {save_beta}
[thread]
n_threads = {chains}
basename = {{DIR}}/out/chain
seeds = {seeds}
[model]
types = {types}
[prior]
use_individual_tau2 = {indiv}
type_A = 1
type_H = 1
type_D = 1
type_R = 1
type_AH = 1
e_qg = {e_qg}
var_qg = {var_qg}
R2mode_sigma2 = 0.2
nu_sigma2 = 1
nu_tau2_A = 5
s2_tau2_A = 0.05
nu_tau2_H = 5
s2_tau2_H = 0.05
nu_tau2_D = 5
eh_tau2_D = 0.1
nu_tau2_R = 5
eh_tau2_R = 0.1
mu_alpha = 1
inv_tau2_e_const_val = 0
inv_tau2_e_val = 0.001
"""


def run_case(name, files, **kw):
    kw.setdefault("efile", "")
    kw.setdefault("yfile", "")
    kw.setdefault("m_e", 0)
    kw.setdefault("recode", 1)
    kw.setdefault("adaptation", 0)
    kw.setdefault("verbosity", 0)
    kw.setdefault("acpt", 0)
    kw.setdefault("nbh", 20)
    kw.setdefault("maxms", 20)
    kw.setdefault("indiv", 0)
    kw.setdefault("dr", 0)
    kw.setdefault("adapt_ms", 1)
    kw.setdefault("flat", 0)
    kw.setdefault("save_beta", 0)
    ini = INI.format(**kw)
    with tempfile.TemporaryDirectory() as d:
        for fn, data in files.items():
            with open(os.path.join(d, fn), "wb") as f:
                f.write(bytes(data))
        os.makedirs(os.path.join(d, "out"))
        ipath = os.path.join(d, "run.ini")
        with open(ipath, "w") as f:
            f.write(ini.replace("{DIR}", d))
        subprocess.run([REF_BIN, ipath], check=True, capture_output=True)
        out = {"ini": np.frombuffer(ini.encode(), dtype=np.uint8)}
        for fn, data in files.items():
            out["file_" + fn.replace(".", "_")] = np.asarray(data, dtype=np.uint8)
        for c in range(kw["chains"]):
            for key, dt in TRACE_FILES.items():
                path = os.path.join(d, "out", "chain%d_%s.dat" % (c, key))
                if os.path.exists(path):
                    out["c%d_%s" % (c, key)] = np.fromfile(path, dtype=dt)
    np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % name), **out)


def with_missing(bed, n, p, frac, seed):
    """A copy of a SNP-major .bed (3-byte magic first) with a seeded fraction
    of the n calls of each of the p SNPs set to the missing code 01."""
    out = np.array(bed, dtype=np.uint8, copy=True)
    stride = (n + 3) // 4
    rng = np.random.default_rng(seed)
    snp, ind = np.nonzero(rng.random((p, n)) < frac)
    pos = 3 + snp * stride + ind // 4
    shift = (2 * (ind % 4)).astype(np.uint8)
    out[pos] = (out[pos] & ~(np.uint8(3) << shift)) | (np.uint8(1) << shift)
    return out


def cases():
    """name -> (files, run_case keywords)"""
    tdir = os.path.join(REF, "src/tests/testdata")
    rd = lambda path: np.frombuffer(open(path, "rb").read(), dtype=np.uint8)
    small = {"data.bed": rd(os.path.join(tdir, "small_modelspace.bed")),
             "data.fam": rd(os.path.join(tdir, "small_modelspace.fam"))}
    # the example dataset (testdata/testdata.ini): first 1500 SNPs, its covariate
    # and alternate phenotype files
    ex = os.path.join(REF, "testdata")
    bed = rd(os.path.join(ex, "testdata.bed"))
    n = 1000
    stride = (n + 3) // 4
    p = 1500
    sub = np.concatenate([bed[:3], bed[3:3 + p * stride]])
    files = {"data.bed": sub, "data.fam": rd(os.path.join(ex, "testdata.fam")),
             "data.e": rd(os.path.join(ex, "testdata.e")), "data.y": rd(os.path.join(ex, "testdata.y"))}
    efiles = dict(efile="file_e = {DIR}/data.e\n", yfile="file_y = {DIR}/data.y\n")
    small_miss = dict(small, **{"data.bed": with_missing(small["data.bed"], 30, 7, 0.05, 11)})
    files_miss = dict(files, **{"data.bed": with_missing(sub, n, p, 0.02, 12)})
    return {
        # the exhaustive-posterior test setting (src/tests/testdata/small_modelspace_tau2.ini),
        # shortened and with delayed rejection off
        "small": (small, dict(n=30, p=7, iters=3000, n_rao=10, burnin=50, thin=5, nst=10,
                              chains=2, seeds="1245,77", types="A", e_qg=2, var_qg=2)),
        "small_types": (small, dict(n=30, p=7, iters=2000, n_rao=10, burnin=20, thin=2, nst=6,
                                    chains=1, seeds="99", types="A,AH", e_qg=2, var_qg=2, indiv=1, maxms=5, nbh=3)),
        # individual tau2, n_rao 10
        "example": (files, dict(n=n, p=p, iters=600, n_rao=10, burnin=20, thin=10, nst=10,
                                chains=2, seeds="1234,2345", types="A", e_qg=20, var_qg=300, m_e=2,
                                indiv=1, verbosity=100, **efiles)),
        "example_types": (files, dict(n=n, p=p, iters=400, n_rao=20, burnin=5, thin=4, nst=8,
                                      chains=1, seeds="4321", types="A,H,D,R,AH", e_qg=20, var_qg=300, m_e=2,
                                      adaptation=1, acpt=0.3, **efiles)),
        # delayed rejection: the small setting with it on (moves of up to 5 SNPs),
        # the example dataset with the example configuration's delay_rejection = 10,
        # and an A,AH case for the left moves of two-column terms
        "small_dr": (small, dict(n=30, p=7, iters=3000, n_rao=10, burnin=50, thin=5, nst=10,
                                 chains=2, seeds="1245,77", types="A", e_qg=2, var_qg=2, maxms=5, dr=5)),
        "example_dr": (files, dict(n=n, p=p, iters=500, n_rao=10, burnin=20, thin=10, nst=10,
                                   chains=2, seeds="1234,2345", types="A", e_qg=20, var_qg=300, m_e=2,
                                   dr=10, **efiles)),
        "small_types_dr": (small, dict(n=30, p=7, iters=2000, n_rao=10, burnin=20, thin=2, nst=6,
                                       chains=1, seeds="99", types="A,AH", e_qg=2, var_qg=2, maxms=5, nbh=3,
                                       dr=5)),
        # missing calls (5 % and 2 % of the calls, seeded): imputation from each
        # SNP's genotype frequencies at every RB step and the Gibbs update of the
        # in-model SNPs' missing calls every nst iterations
        "small_types_missing": (small_miss, dict(n=30, p=7, iters=2000, n_rao=10, burnin=20, thin=2, nst=6,
                                                 chains=1, seeds="99", types="A,AH", e_qg=2, var_qg=2, indiv=1,
                                                 maxms=5, nbh=3)),
        # a flat proposal (no RB-adapted add weights), the beta trace, raw
        # (not minor-allele recoded) genotypes and a fixed move-size distribution
        "small_flat": (small, dict(n=30, p=7, iters=2000, n_rao=10, burnin=20, thin=2, nst=6, chains=2,
                                   seeds="5,6", types="A", e_qg=2, var_qg=2, flat=1, save_beta=1, recode=0,
                                   adapt_ms=0)),
        "example_flat": (files, dict(n=n, p=p, iters=400, n_rao=10, burnin=20, thin=10, nst=10, chains=1,
                                     seeds="31", types="A,AH", e_qg=20, var_qg=300, m_e=2, flat=1, save_beta=1,
                                     **efiles)),
        # the features together: missing calls, two effect types, delayed
        # rejection and continued adaptation with an acceptance-rate goal
        "small_types_dr_missing": (small_miss, dict(n=30, p=7, iters=2000, n_rao=10, burnin=20, thin=2, nst=6,
                                                    chains=2, seeds="3,4", types="A,AH", e_qg=2, var_qg=2,
                                                    indiv=1, maxms=5, nbh=3, dr=5, adaptation=1, acpt=0.3)),
        # individual tau2 with all five effect types: the scan's per-SNP tau2
        # draws then cover four terms
        "example_types_indiv": (files, dict(n=n, p=p, iters=300, n_rao=10, burnin=5, thin=5, nst=8, chains=1,
                                            seeds="23", types="A,H,D,R,AH", e_qg=20, var_qg=300, m_e=2, indiv=1,
                                            **efiles)),
        # a prior that puts most mass on ~600 of the 1500 SNPs: the model grows
        # past 128 columns (A,AH terms), where the GPU keeps its Cholesky
        # factors in global memory instead of shared memory
        "example_large": (files, dict(n=n, p=p, iters=300, n_rao=10, burnin=10, thin=5, nst=10, chains=1,
                                      seeds="17", types="A,AH", e_qg=600, var_qg=2000, m_e=2, **efiles)),
        "example_missing": (files_miss, dict(n=n, p=p, iters=600, n_rao=10, burnin=20, thin=10, nst=10,
                                             chains=2, seeds="1234,2345", types="A", e_qg=20, var_qg=300, m_e=2,
                                             indiv=1, **efiles)),
    }


def edit_ini(text, section, key, value):
    """Set (or with value None delete) one key of an INI text; a key that is
    absent is added at the top of its section."""
    pat = re.compile(r"(?m)^%s\s*[=:].*$" % re.escape(key))
    if pat.search(text):
        return pat.sub("" if value is None else "%s = %s" % (key, value), text)
    if value is None:
        return text
    return text.replace("[%s]\n" % section, "[%s]\n%s = %s\n" % (section, key, value), 1)


# edits of the example configuration (testdata/testdata.ini): one rule of the
# reference's parser (src/options.hpp:138-321) each
OPTION_EDITS = {
    "example": [],
    "types_unsorted": [("model", "types", "H, A, AH")],
    "types_all": [("model", "types", "AH,R,D,H,A"), ("prior", "nu_tau2_D", "4"), ("prior", "eh_tau2_D", "0.2"),
                  ("prior", "nu_tau2_R", "3"), ("prior", "s2_tau2_R", "0.01")],
    "types_unknown": [("model", "types", "A, Q")],
    "types_empty": [("model", "types", "")],
    "types_missing_prior": [("model", "types", "A, R")],
    "thin_not_divisor": [("sampler", "thin", "3")],
    "defaults": [("sampler", k, None) for k in ("max_move_size", "p_move_size", "p_move_size_nbc", "p_move_size_nbs",
                                               "max_SNP_neighborhood_size", "adapt_p_move_size",
                                               "p_move_size_acpt_goal", "flat_proposal_dist", "delay_rejection",
                                               "adaptation", "type")] +
                [("thread", "basename", None), ("prior", "use_individual_tau2", None), ("prior", "type_AH", None),
                 ("prior", "mu_alpha", None)],
    "p_move_size_above_1": [("sampler", "p_move_size", "1.5")],
    "p_move_size_nbs_zero": [("sampler", "p_move_size_nbs", "0")],
    "acpt_goal": [("sampler", "p_move_size_acpt_goal", "0.3")],
    "acpt_goal_above_1": [("sampler", "p_move_size_acpt_goal", "1.2")],
    "seeds_short": [("thread", "n_threads", "3")],
    "seeds_repeated": [("thread", "seeds", "7, 7")],
    "sampler_unknown": [("sampler", "type", "XYZ")],
    "sampler_nk_ah": [("sampler", "type", "NK"), ("model", "types", "A, AH")],
    "bool_bad": [("sampler", "adaptation", "2")],
    "bool_words": [("sampler", "adaptation", "true"), ("sampler", "flat_proposal_dist", "no")],
    "r2mode_bad": [("prior", "R2mode_sigma2", "1.5")],
    "s2_sigma2_given": [("prior", "R2mode_sigma2", None), ("prior", "s2_sigma2", "0.5")],
    "nu_sigma2_negative": [("prior", "nu_sigma2", "-1")],
    "n_missing": [("sizes", "n", None)],
    "n_not_integer": [("sizes", "n", "12x")],
    "n_zero": [("sizes", "n", "0")],
    "no_covariates": [("sizes", "m_e", "0"), ("datafiles", "file_e", None)],
    "covariates_without_file": [("datafiles", "file_e", None)],
    "eh_tau2": [("prior", "s2_tau2_A", None), ("prior", "eh_tau2_A", "0.1")],
    "shared_tau2": [("prior", "use_individual_tau2", "0"), ("prior", "inv_tau2_e_const_val", "0.5")],
    "no_y_file": [("datafiles", "file_y", None)],
    "recode_off": [("datafiles", "recode_g_to_minor_allele_count", "0")],
    "verbosity_missing": [("sampler", "verbosity", None)],
    "burnin_zero": [("sampler", "n_rao_burnin", "0")],
}


def option_cases():
    """INI texts for the parser parity fixture: the reference's own INI files
    and the edits of OPTION_EDITS."""
    out = {}
    example = open(os.path.join(REF, "testdata", "testdata.ini")).read()
    for name, edits in OPTION_EDITS.items():
        text = example
        for section, key, value in edits:
            text = edit_ini(text, section, key, value)
        out[name] = text
    tdir = os.path.join(REF, "src", "tests", "testdata")
    for f in sorted(os.listdir(tdir)):
        if f.endswith(".ini"):
            out["tests_" + f[:-4]] = open(os.path.join(tdir, f)).read()
    return out


def options_fixture():
    """Run the reference's option parser (oracle/_ref/ref_probe) over every
    case; store each INI text with the parsed fields (or the error) and the
    warnings it printed, in order."""
    cases = []
    with tempfile.TemporaryDirectory() as d:
        for name, text in option_cases().items():
            path = os.path.join(d, "opt.ini")
            with open(path, "w") as f:
                f.write(text)
            r = subprocess.run([REF_PROBE, path], check=True, capture_output=True, text=True)
            fields, warnings = {}, []
            for line in r.stdout.splitlines():
                if line.startswith("opt."):
                    k, v = line[4:].split("=", 1)
                    fields[k] = v
                elif line.startswith("Warning"):
                    warnings.append(line)
            cases.append({"name": name, "ini": text, "fields": fields, "warnings": warnings})
    with open(os.path.join(HERE, "options_ref.json"), "w") as f:
        json.dump(cases, f, indent=0, sort_keys=True)


READER_INI = """[datafiles]
file_fam = {DIR}/d.fam
file_g = {DIR}/d.bed
recode_g_to_minor_allele_count = 1
%s
[sizes]
n = 11
m_g = 4
m_e = %d
[sampler]
do_n_iter = 10
n_rao = 10
n_rao_burnin = 1
thin = 1
n_sample_tau2_and_missing = 10
verbosity = 0
[thread]
n_threads = 1
seeds = 5
[model]
types = A
[prior]
e_qg = 1
var_qg = 1
nu_sigma2 = 1
R2mode_sigma2 = 0.2
nu_tau2_A = 5
s2_tau2_A = 0.05
mu_alpha = 1
inv_tau2_e_const_val = 0
inv_tau2_e_val = 0.001
"""


def reader_cases():
    """Input files of the reader parity fixture: n = 11 individuals, 4 SNPs,
    two covariates, and one edit per reader rule of src/data.cpp:141-273.
    A .fam with more than n rows is left out: the reference writes past the
    end of its phenotype vector before it checks the count (src/data.cpp:158)."""
    rng = np.random.default_rng(21)
    n, p = 11, 4
    ids = [("F%d" % (i // 3), "I%d" % i) for i in range(n)]
    g = rng.integers(0, 3, size=(p, n))
    code = np.where(g == 0, 0, np.where(g == 1, 2, 3)).astype(np.uint8)
    pad = np.zeros((p, 12), dtype=np.uint8)
    pad[:, :n] = code
    pad = pad.reshape(p, 3, 4)
    body = (pad[..., 0] | pad[..., 1] << 2 | pad[..., 2] << 4 | pad[..., 3] << 6).astype(np.uint8).reshape(-1)
    bed = bytes([0x6C, 0x1B, 0x01]) + body.tobytes()
    y = np.round(rng.normal(size=n), 6)
    yalt = np.round(rng.normal(size=n), 6)
    ecov = np.round(rng.normal(size=(n, 2)), 6)
    order = rng.permutation(n)
    fam_rows = ["%s %s 0 0 %d %.17g" % (f, i, 1 + k % 2, y[k]) for k, (f, i) in enumerate(ids)]
    y_rows = ["%s %s %.17g" % (ids[k][0], ids[k][1], yalt[k]) for k in order]
    e_rows = ["%s %s %.17g %.17g" % (ids[k][0], ids[k][1], ecov[k, 0], ecov[k, 1]) for k in order]
    join = lambda rows: "\n".join(rows) + "\n"
    base = {"d.fam": join(fam_rows), "d.y": join(y_rows + ["nobody nobody 1.5"]), "d.e": join(e_rows),
            "d.bed": bed}
    edit = lambda **kw: dict(base, **kw)
    fam_tab = [r.replace(" ", "\t", 2) for r in fam_rows]
    cases = {
        "base": (base, True, True),
        "no_alternate_files": (base, False, False),
        "fam_no_trailing_newline": (edit(**{"d.fam": "\n".join(fam_rows)}), True, True),
        "fam_tabs": (edit(**{"d.fam": join(fam_tab)}), True, True),
        "fam_minus_9": (edit(**{"d.fam": join(fam_rows[:3] + ["F1 I3 0 0 1 -9"] + fam_rows[4:])}), False, False),
        "fam_na": (edit(**{"d.fam": join(fam_rows[:5] + ["F1 I5 0 0 1 NA"] + fam_rows[6:])}), False, False),
        "fam_duplicate": (edit(**{"d.fam": join(fam_rows[:10] + [fam_rows[9]])}), False, False),
        "fam_short": (edit(**{"d.fam": join(fam_rows[:-1])}), False, False),
        "y_missing_row": (edit(**{"d.y": join(y_rows[1:])}), True, False),
        "y_no_trailing_newline": (edit(**{"d.y": "\n".join(y_rows)}), True, False),
        "y_extra_column": (edit(**{"d.y": join([y_rows[0] + " 7"] + y_rows[1:])}), True, False),
        "y_duplicate_row": (edit(**{"d.y": join(y_rows + [y_rows[0]])}), True, False),
        "e_nan_first": (edit(**{"d.e": join(["%s %s nan 1.0" % ids[0]] + e_rows)}), False, True),
        "e_nan_last": (edit(**{"d.e": join(e_rows + ["%s %s nan 1.0" % ids[0]])}), False, True),
        "e_short_row": (edit(**{"d.e": join([" ".join(e_rows[0].split()[:3])] + e_rows[1:])}), False, True),
        "e_unknown_row": (edit(**{"d.e": join(["X Y 1 2"] + e_rows)}), False, True),
        "bed_bad_magic": (edit(**{"d.bed": bytes([0x6C, 0x1C, 0x01]) + body.tobytes()}), False, False),
        "bed_individual_major": (edit(**{"d.bed": bytes([0x6C, 0x1B, 0x00]) + body.tobytes()}), False, False),
        "bed_short": (edit(**{"d.bed": bed[:-1]}), False, False),
        "bed_longer": (edit(**{"d.bed": bed + bytes([0xFF, 0x00])}), False, False),
    }
    return cases


def readers_fixture():
    """Run the reference's Data class (oracle/_ref/ref_probe --data) on each
    reader case; store the files (the .bed base64-encoded), the INI and what
    it read (phenotypes, covariates, summary statistics) or its error."""
    out = []
    with tempfile.TemporaryDirectory() as d:
        for name, (files, with_y, with_e) in reader_cases().items():
            extra = ("file_y = {DIR}/d.y\n" if with_y else "") + ("file_e = {DIR}/d.e\n" if with_e else "")
            ini = READER_INI % (extra, 2 if with_e else 0)
            for fn, data in files.items():
                with open(os.path.join(d, fn), "wb") as f:
                    f.write(data if isinstance(data, bytes) else data.encode())
            with open(os.path.join(d, "r.ini"), "w") as f:
                f.write(ini.replace("{DIR}", d))
            r = subprocess.run([REF_PROBE, "--data", os.path.join(d, "r.ini")], check=True, capture_output=True,
                               text=True)
            if "opt.error=" in r.stdout:
                raise SystemExit("reader case %s: %s" % (name, r.stdout.split("opt.error=")[1].strip()))
            res = dict(line[5:].split("=", 1) for line in r.stdout.splitlines() if line.startswith("data."))
            enc = {fn: (base64.b64encode(v).decode() if isinstance(v, bytes) else v) for fn, v in files.items()}
            out.append({"name": name, "ini": ini, "files": enc, "result": res})
    with open(os.path.join(HERE, "readers_ref.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)


def main():
    if not os.path.exists(REF_BIN):
        raise SystemExit("build oracle/_ref first (make -C oracle)")
    names = sys.argv[2:]
    if not names:
        known_answers()
    if not names or "options" in names:
        options_fixture()
    if not names or "readers" in names:
        readers_fixture()
    for name, (files, kw) in cases().items():
        if names and name not in names:
            continue
        run_case(name, files, **kw)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
