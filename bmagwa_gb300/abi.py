"""ctypes mirror of include/bmg.h (the C ABI of libbmg).

The structures here are laid out field for field like the C header; every
entry point of the library is bound with its argument types so a wrong call
fails in Python instead of in native code.
"""
import ctypes as C
import os

MAX_PATH = 1024

BMG_OK = 0
STATUS_NAMES = {
    0: "BMG_OK", 1: "BMG_EINVAL", 2: "BMG_EIO", 3: "BMG_ECUDA", 4: "BMG_ENOTPD",
    5: "BMG_ETIMEOUT", 6: "BMG_ENOMEM", 7: "BMG_EUNSUPPORTED", 8: "BMG_ENUMERIC",
}

TYPE_A, TYPE_H, TYPE_D, TYPE_R, TYPE_AH = 0, 1, 2, 3, 4
TYPE_NAMES = {"A": TYPE_A, "H": TYPE_H, "D": TYPE_D, "R": TYPE_R, "AH": TYPE_AH}
PROPOSAL_ADAPTIVE, PROPOSAL_LEARNED = 0, 1
SCAN_TCGEN05, SCAN_SIMT = 0, 1


class Options(C.Structure):
    _fields_ = [
        ("file_fam", C.c_char * MAX_PATH),
        ("file_g", C.c_char * MAX_PATH),
        ("file_e", C.c_char * MAX_PATH),
        ("file_y", C.c_char * MAX_PATH),
        ("recode_g_to_minor_allele_count", C.c_int32),
        ("n", C.c_uint64),
        ("m_g", C.c_uint64),
        ("m_e", C.c_uint32),
        ("n_types", C.c_uint32),
        ("types", C.c_int32 * 5),
        ("sampler_type", C.c_int32),
        ("do_n_iter", C.c_uint64),
        ("n_rao", C.c_uint64),
        ("n_rao_burnin", C.c_uint64),
        ("thin", C.c_uint64),
        ("n_sample_tau2_and_missing", C.c_uint64),
        ("max_move_size", C.c_uint32),
        ("max_SNP_neighborhood_size", C.c_uint32),
        ("p_move_size", C.c_double),
        ("p_move_size_nbs", C.c_double),
        ("p_move_size_nbc", C.c_double),
        ("adapt_p_move_size", C.c_int32),
        ("p_move_size_acpt_goal", C.c_double),
        ("adaptation", C.c_int32),
        ("flat_proposal_dist", C.c_int32),
        ("save_beta", C.c_int32),
        ("verbosity", C.c_uint64),
        ("delay_rejection", C.c_uint32),
        ("basename", C.c_char * MAX_PATH),
        ("n_chains", C.c_uint32),
        ("seeds", C.POINTER(C.c_uint32)),
        ("e_qg", C.c_double),
        ("var_qg", C.c_double),
        ("nu_sigma2", C.c_double),
        ("s2_sigma2", C.c_double),
        ("R2mode_sigma2", C.c_double),
        ("mu_alpha", C.c_double),
        ("inv_tau2_e_const_val", C.c_double),
        ("inv_tau2_e_val", C.c_double),
        ("use_individual_tau2", C.c_int32),
        ("types_prior", C.c_double * 5),
        ("nu_tau2", C.c_double * 4),
        ("s2_tau2", C.c_double * 4),
        ("eh_tau2", C.c_double * 4),
        ("max_model_size", C.c_uint32),
        ("scan_limbs", C.c_uint32),
        ("scan_impl", C.c_int32),
        ("proposal", C.c_int32),
        ("graph_iters", C.c_uint32),
        ("write_files", C.c_int32),
        ("quiet", C.c_int32),
        ("learned_mix", C.c_double),
        ("learned_topk", C.c_uint32),
        ("learned_every", C.c_uint32),
        ("learned_steps", C.c_uint32),
        ("learned_lr", C.c_double),
    ]


class TraceChunk(C.Structure):
    _fields_ = [
        ("chain", C.c_uint32),
        ("iter0", C.c_uint64),
        ("n_iter", C.c_uint64),
        ("jumpdistance", C.POINTER(C.c_uint8)),
        ("move_type", C.POINTER(C.c_uint8)),
        ("move_size", C.POINTER(C.c_uint8)),
        ("n_thin", C.c_uint64),
        ("modelsize", C.POINTER(C.c_uint32)),
        ("n_loci", C.c_uint64),
        ("loci", C.POINTER(C.c_uint32)),
        ("types", C.POINTER(C.c_uint8)),
        ("log_likelihood", C.POINTER(C.c_double)),
        ("log_prior", C.POINTER(C.c_double)),
        ("sigma2", C.POINTER(C.c_double)),
        ("alpha", C.POINTER(C.c_double)),
        ("pve", C.POINTER(C.c_double)),
        ("n_beta", C.c_uint64),
        ("beta", C.POINTER(C.c_double)),
    ]


TRACE_FN = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(TraceChunk))


class TraceSink(C.Structure):
    _fields_ = [("fn", TRACE_FN), ("user", C.c_void_p)]


class ChainState(C.Structure):
    _fields_ = [
        ("model_size", C.c_uint32),
        ("log_likelihood", C.c_double),
        ("log_prior", C.c_double),
        ("sigma2", C.c_double),
        ("alpha", C.c_double),
        ("n_iter", C.c_uint64),
        ("n_accepted", C.c_uint64),
        ("p_move_size", C.c_double),
        ("rng_draws", C.c_uint64),
    ]


def _arr(ptr, n, dtype):
    import numpy as np
    if n == 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(int(n),)).astype(dtype, copy=True)


class TraceCollector:
    """Accumulates bmg_trace_chunk callbacks per chain into numpy arrays."""

    KEYS = ("jumpdistance", "move_type", "move_size", "modelsize", "loci", "types",
            "log_likelihood", "log_prior", "sigma2", "alpha", "pve", "beta")

    def __init__(self):
        self.parts = {}
        self._cb = TRACE_FN(self._on_chunk)
        self.sink = TraceSink(self._cb, None)

    def _on_chunk(self, _user, chunk_p):
        import numpy as np
        k = chunk_p.contents
        d = self.parts.setdefault(k.chain, {key: [] for key in self.KEYS})
        d["jumpdistance"].append(_arr(k.jumpdistance, k.n_iter, np.uint8))
        d["move_type"].append(_arr(k.move_type, k.n_iter, np.uint8))
        d["move_size"].append(_arr(k.move_size, k.n_iter, np.uint8))
        d["modelsize"].append(_arr(k.modelsize, k.n_thin, np.uint32))
        d["loci"].append(_arr(k.loci, k.n_loci, np.uint32))
        d["types"].append(_arr(k.types, k.n_loci if k.types else 0, np.uint8))
        d["log_likelihood"].append(_arr(k.log_likelihood, k.n_thin, np.float64))
        d["log_prior"].append(_arr(k.log_prior, k.n_thin, np.float64))
        d["sigma2"].append(_arr(k.sigma2, k.n_thin, np.float64))
        d["alpha"].append(_arr(k.alpha, k.n_thin, np.float64))
        d["pve"].append(_arr(k.pve, 3 * k.n_thin, np.float64))
        d["beta"].append(_arr(k.beta, k.n_beta, np.float64))

    def chain(self, c):
        import numpy as np
        d = self.parts.get(c)
        if d is None:
            return None
        return {key: (np.concatenate(v) if v else np.zeros(0)) for key, v in d.items()}


def set_path(opt, field, value):
    b = os.fsencode(value)
    if len(b) >= MAX_PATH:
        raise ValueError("path too long")
    setattr(opt, field, b)


def default_options():
    """The reference's defaults of every optional key (src/options.hpp:138-321)
    and the library's defaults of its own knobs, filled without loading the
    library: the same values bmg_options_default() writes (a CPU test checks
    them field by field), for callers that drive only the oracle."""
    o = Options()
    o.sampler_type = 0
    o.max_move_size = 20
    o.max_SNP_neighborhood_size = 10
    o.p_move_size = o.p_move_size_nbs = o.p_move_size_nbc = 0.2
    o.adapt_p_move_size = 1
    o.p_move_size_acpt_goal = 0.0
    o.basename = b"chain"
    o.n_chains = 1
    for t in range(5):
        o.types_prior[t] = 1.0
    o.max_model_size = 1024
    o.scan_limbs = 6
    o.scan_impl = SCAN_TCGEN05
    o.proposal = PROPOSAL_ADAPTIVE
    o.graph_iters = 64
    o.learned_mix = 0.3
    o.learned_topk = 1024
    o.learned_every = 10
    o.learned_steps = 4
    o.learned_lr = 1e-3
    return o


def set_seeds(opt, seeds):
    """Point opt.seeds at a new array of the given seeds (kept alive with the struct)."""
    arr = (C.c_uint32 * len(seeds))(*[int(s) for s in seeds])
    opt.seeds = C.cast(arr, C.POINTER(C.c_uint32))
    opt.n_chains = len(seeds)
    opt._seeds = arr
    return opt


def bind_common(lib):
    """Argument types of the entry points that need no device."""
    lib.bmg_options_default.argtypes = [C.POINTER(Options)]
    lib.bmg_options_default.restype = C.c_int
    lib.bmg_options_from_ini.argtypes = [C.c_char_p, C.POINTER(Options), C.POINTER(C.c_uint32),
                                         C.c_uint32, C.c_char_p, C.c_size_t]
    lib.bmg_options_from_ini.restype = C.c_int
    lib.bmg_read_plink.argtypes = [C.POINTER(Options), C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_char_p, C.c_size_t]
    lib.bmg_read_plink.restype = C.c_int
