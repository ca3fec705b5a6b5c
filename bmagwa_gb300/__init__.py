"""bmagwa_gb300: GB300 (sm_103a) build of bmagwa's MCMC over SNP inclusion.

Python handle on libbmg (include/bmg.h).  The reference's entry points map as:

    bmagwa INIFILE               -> run_ini(path)  /  bmagwa-gb300 INIFILE
    bmagwa::Options(ini)         -> options_from_ini(path)
    bmagwa::Data(...)            -> read_plink(opt) + Context.load_bed /
                                    set_phenotypes / set_covariates
    PrecomputedSNPCovariances    -> Context.precompute()
    Sampler::sample()            -> Context.run(n_iter)
    RaoBlackwellizer             -> Context.scan()

Every call goes to the CUDA library; there is no CPU fallback.  If the
library is not built, importing works but the first call raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

__all__ = ["lib", "options_from_ini", "default_options", "read_plink", "Context", "run_ini",
           "BmgError", "build"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libbmg.so")
_lib = None


class BmgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, status), msg))
        self.status = status


def build(force=False, verbose=False):
    from . import nvbuild as _b
    return _b.build(force=force, verbose=verbose)


def lib():
    """The loaded libbmg (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libbmg is not built (run bmagwa_gb300.build() or __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        abi.bind_common(L)
        vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
        L.bmg_create.argtypes = [C.POINTER(abi.Options), C.POINTER(vp)]
        L.bmg_load_bed.argtypes = [vp, vp, u64, u64]
        L.bmg_set_phenotypes.argtypes = [vp, vp, vp, u32]
        L.bmg_set_covariates.argtypes = [vp, vp, u32]
        L.bmg_precompute.argtypes = [vp]
        L.bmg_get_precomputed.argtypes = [vp, vp, C.POINTER(u32)]
        L.bmg_scan.argtypes = [vp, vp, vp]
        L.bmg_scan_logodds.argtypes = [vp, vp]
        L.bmg_scan_schur.argtypes = [vp, vp]
        L.bmg_learned_snapshot.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.bmg_learned_grad.argtypes = [vp, vp, u32, vp]
        L.bmg_run.argtypes = [vp, u64, C.POINTER(abi.TraceSink)]
        L.bmg_get_state.argtypes = [vp, u32, C.POINTER(abi.ChainState), vp, vp, u32]
        L.bmg_get_rao.argtypes = [vp, u32, vp, vp]
        L.bmg_get_rao_all.argtypes = [vp, vp, vp]
        L.bmg_finish.argtypes = [vp]
        L.bmg_get_timings.argtypes = [vp, vp]
        L.bmg_get_proposal.argtypes = [vp, u32, vp, vp]
        L.bmg_reset_timings.argtypes = [vp, C.POINTER(u64)]
        L.bmg_precompute_noalloc.argtypes = [vp, u64, u64, C.c_int32, C.POINTER(C.c_int32), u32, vp,
                                             C.POINTER(u32), vp, vp]
        L.bmg_precompute_noalloc.restype = C.c_int
        L.bmg_scan_yhat.argtypes = [vp, vp, C.c_double, vp, vp]
        L.bmg_scan_yhat.restype = C.c_int
        L.bmg_get_last_scan.argtypes = [vp, u32, vp, vp]
        L.bmg_get_data_stats.argtypes = [vp, vp]
        L.bmg_get_launch_count.argtypes = [vp, C.POINTER(u64)]
        L.bmg_selftest_exp.argtypes = [vp, vp, C.c_size_t]
        L.bmg_selftest_exp.restype = C.c_int
        L.bmg_get_scan_shape.argtypes = [vp, C.POINTER(C.c_int32), C.c_char_p, C.c_size_t]
        L.bmg_get_scan_tuning.argtypes = [vp, vp, C.c_int32, C.POINTER(C.c_int32)]
        L.bmg_get_scan_tuning.restype = C.c_int
        L.bmg_get_scan_shape_name.argtypes = [C.c_int32, C.c_char_p, C.c_size_t]
        L.bmg_get_scan_shape_name.restype = C.c_int
        L.bmg_last_error.argtypes = [vp]
        L.bmg_last_error.restype = C.c_char_p
        L.bmg_status_string.argtypes = [C.c_int]
        L.bmg_status_string.restype = C.c_char_p
        L.bmg_destroy.argtypes = [vp]
        L.bmg_destroy.restype = None
        for name in ("bmg_create", "bmg_load_bed", "bmg_set_phenotypes", "bmg_set_covariates",
                     "bmg_precompute", "bmg_get_precomputed", "bmg_scan", "bmg_run", "bmg_get_state",
                     "bmg_get_rao", "bmg_get_rao_all", "bmg_finish", "bmg_get_timings", "bmg_get_data_stats",
                     "bmg_get_proposal", "bmg_get_last_scan", "bmg_reset_timings"):
            getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def default_options():
    o = abi.Options()
    lib().bmg_options_default(C.byref(o))
    return o


def options_from_ini(path, quiet=True):
    """Parse a reference INI file; returns (options, seeds array)."""
    o = abi.Options()
    o.quiet = 1 if quiet else 0
    seeds = (C.c_uint32 * 4096)()
    err = C.create_string_buffer(1024)
    rc = lib().bmg_options_from_ini(os.fsencode(path), C.byref(o), seeds, 4096, err, 1024)
    if rc != 0:
        raise BmgError(rc, err.value.decode())
    o._seeds = seeds  # keep the buffer alive with the struct
    return o


def set_seeds(opt, seeds):
    return abi.set_seeds(opt, seeds)


def read_plink(opt):
    """Read the .fam/.bed (and .y/.e) files an options struct names."""
    n, p, me = int(opt.n), int(opt.m_g), int(opt.m_e)
    packed = np.zeros(p * ((n + 3) // 4), dtype=np.uint8)
    y = np.zeros(n)
    e = np.zeros(n * me) if me else None
    err = C.create_string_buffer(1024)
    rc = lib().bmg_read_plink(C.byref(opt), _ptr(packed), _ptr(y), _ptr(e), err, 1024)
    if rc != 0:
        raise BmgError(rc, err.value.decode())
    return packed, y, e


class Context:
    """All chains of one options struct on one dataset, on the current GPU."""

    def __init__(self, opt):
        self.opt = opt
        self.n = int(opt.n)
        self.m_g = int(opt.m_g)
        self.n_types = int(opt.n_types)
        self.n_chains = int(opt.n_chains)
        terms = set()
        for i in range(int(opt.n_types)):
            t = int(opt.types[i])
            terms.update((0, 1) if t == 4 else (t,))
        self.n_terms = len(terms)
        h = C.c_void_p()
        rc = lib().bmg_create(C.byref(opt), C.byref(h))
        if rc != 0:
            raise BmgError(rc, lib().bmg_last_error(None).decode())
        self.h = h

    def _check(self, rc):
        if rc != 0:
            raise BmgError(rc, lib().bmg_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            lib().bmg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_bed(self, packed):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        self._check(lib().bmg_load_bed(self.h, _ptr(packed), int(self.opt.n), self.m_g))

    def set_phenotypes(self, y, mask=None):
        y = np.ascontiguousarray(y, dtype=np.float64)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        n_pheno = 1 if y.ndim == 1 else y.shape[0]
        self._check(lib().bmg_set_phenotypes(self.h, _ptr(y), _ptr(m), n_pheno))

    def set_covariates(self, e):
        if e is None:
            self._check(lib().bmg_set_covariates(self.h, None, 0))
            return
        e = np.ascontiguousarray(e, dtype=np.float64).reshape(-1)
        self._check(lib().bmg_set_covariates(self.h, _ptr(e), int(self.opt.m_e)))

    def precompute(self):
        self._check(lib().bmg_precompute(self.h))

    def precomputed(self):
        off = C.c_uint32()
        self._check(lib().bmg_get_precomputed(self.h, None, C.byref(off)))
        xx = np.zeros(self.m_g * off.value)
        self._check(lib().bmg_get_precomputed(self.h, _ptr(xx), C.byref(off)))
        return xx.reshape(self.m_g, off.value)

    def run(self, n_iter, collect=True):
        col = abi.TraceCollector() if collect else None
        sink = C.byref(col.sink) if col else None
        self._check(lib().bmg_run(self.h, int(n_iter), sink))
        return col

    def scan(self):
        pr = np.zeros(self.n_chains * self.m_g)
        prt = np.zeros(self.n_chains * self.m_g * self.n_types) if self.n_types > 1 else None
        self._check(lib().bmg_scan(self.h, _ptr(pr), _ptr(prt)))
        pr = pr.reshape(self.n_chains, self.m_g)
        if prt is not None:
            prt = prt.reshape(self.n_chains, self.m_g, self.n_types)
        return pr, prt

    def scan_logodds(self):
        """(chains, m_g) per-SNP log posterior odds of inclusion of an RB scan
        of every chain's current state."""
        lo = np.zeros(self.n_chains * self.m_g)
        self._check(lib().bmg_scan_logodds(self.h, _ptr(lo)))
        return lo.reshape(self.n_chains, self.m_g)

    def scan_yhat(self, y_hat, sigma2):
        """RB scan of every chain against the given fitted values (n doubles)
        and sigma2 (which becomes every chain's sigma2): (p_r, log odds), each
        (chains, m_g)."""
        yh = np.ascontiguousarray(y_hat, dtype=np.float64)
        if yh.size != self.n:
            raise ValueError("y_hat must have n entries")
        pr = np.zeros(self.n_chains * self.m_g)
        lo = np.zeros(self.n_chains * self.m_g)
        self._check(lib().bmg_scan_yhat(self.h, _ptr(yh), float(sigma2), _ptr(pr), _ptr(lo)))
        return pr.reshape(self.n_chains, self.m_g), lo.reshape(self.n_chains, self.m_g)

    def scan_schur(self):
        """(chains, m_g, terms) exact change of each chain's log marginal
        likelihood from adding each single term of each SNP outside its model."""
        nt = self.n_terms
        out = np.zeros(self.n_chains * self.m_g * nt)
        self._check(lib().bmg_scan_schur(self.h, _ptr(out)))
        return out.reshape(self.n_chains, self.m_g, nt)

    MLP_NPAR = 18817

    def learned_snapshot(self, features=False):
        """(theta, logits (chains, m_g), features (chains, m_g, 16) or None,
        tables: list of (snps, weights) per chain) of the learned proposal."""
        C_, p = self.n_chains, self.m_g
        topk = int(self.opt.learned_topk)
        th = np.zeros(self.MLP_NPAR, dtype=np.float32)
        lg = np.zeros(C_ * p, dtype=np.float32)
        ft = np.zeros(C_ * p * 16, dtype=np.float32) if features else None
        ts = np.zeros(C_ * topk, dtype=np.uint32)
        tw = np.zeros(C_ * topk)
        tn = np.zeros(C_, dtype=np.uint32)
        self._check(lib().bmg_learned_snapshot(self.h, _ptr(th), _ptr(lg), _ptr(ft), _ptr(ts), _ptr(tw), _ptr(tn)))
        tables = [(ts[c * topk:c * topk + tn[c]].copy(), tw[c * topk:c * topk + tn[c]].copy()) for c in range(C_)]
        return th, lg.reshape(C_, p), (ft.reshape(C_, p, 16) if features else None), tables

    def learned_grad(self, rows):
        """Gradient of the training loss over rows [(chain, snp), ...]."""
        r = np.ascontiguousarray(np.asarray(rows, dtype=np.uint32).reshape(-1, 2))
        g = np.zeros(self.MLP_NPAR, dtype=np.float32)
        self._check(lib().bmg_learned_grad(self.h, _ptr(r), len(r), _ptr(g)))
        return g

    def state(self, chain=0, cap=4096):
        st = abi.ChainState()
        loci = np.zeros(cap, dtype=np.uint32)
        types = np.zeros(cap, dtype=np.uint8)
        self._check(lib().bmg_get_state(self.h, chain, C.byref(st), _ptr(loci), _ptr(types), cap))
        k = st.model_size
        return st, loci[:k].copy(), types[:k].copy()

    def rao(self, chain=0):
        p = np.zeros(self.m_g)
        pt = np.zeros(self.m_g * self.n_types) if self.n_types > 1 else None
        self._check(lib().bmg_get_rao(self.h, chain, _ptr(p), _ptr(pt)))
        return p, (pt.reshape(self.m_g, self.n_types) if pt is not None else None)

    def rao_all(self):
        """Rao-Blackwellised posteriors of every chain in one call:
        (chains x m_g, chains x m_g x n_types or None)."""
        p = np.zeros(self.opt.n_chains * self.m_g)
        pt = np.zeros(self.opt.n_chains * self.m_g * self.n_types) if self.n_types > 1 else None
        self._check(lib().bmg_get_rao_all(self.h, _ptr(p), _ptr(pt)))
        return (p.reshape(self.opt.n_chains, self.m_g),
                pt.reshape(self.opt.n_chains, self.m_g, self.n_types) if pt is not None else None)

    def proposal(self, chain=0):
        p = np.zeros(self.m_g)
        pt = np.zeros(self.m_g * self.n_types) if self.n_types > 1 else None
        self._check(lib().bmg_get_proposal(self.h, chain, _ptr(p), _ptr(pt)))
        return p, (pt.reshape(self.m_g, self.n_types) if pt is not None else None)

    def last_scan(self, chain=0):
        p = np.zeros(self.m_g)
        pt = np.zeros(self.m_g * self.n_types) if self.n_types > 1 else None
        self._check(lib().bmg_get_last_scan(self.h, chain, _ptr(p), _ptr(pt)))
        return p, (pt.reshape(self.m_g, self.n_types) if pt is not None else None)

    def data_stats(self):
        out = np.zeros(4)
        self._check(lib().bmg_get_data_stats(self.h, _ptr(out)))
        return out

    def timings(self):
        out = np.zeros(4)
        self._check(lib().bmg_get_timings(self.h, _ptr(out)))
        return out

    def launch_count(self):
        """Kernels launched since the last reset_timings()."""
        n = C.c_uint64(0)
        self._check(lib().bmg_get_launch_count(self.h, C.byref(n)))
        return int(n.value)

    def scan_shape(self):
        """(variant, description) of the tensor-core scan's launch shape."""
        v = C.c_int32(-1)
        buf = C.create_string_buffer(128)
        self._check(lib().bmg_get_scan_shape(self.h, C.byref(v), buf, 128))
        return int(v.value), buf.value.decode()

    def scan_tuning(self):
        """{shape description: fastest tuning scan in ms} of the scan's tuner."""
        n = C.c_int32(0)
        self._check(lib().bmg_get_scan_tuning(self.h, None, 0, C.byref(n)))
        ms = np.zeros(n.value, dtype=np.float32)
        self._check(lib().bmg_get_scan_tuning(self.h, _ptr(ms), n.value, None))
        out = {}
        for i in range(n.value):
            buf = C.create_string_buffer(128)
            self._check(lib().bmg_get_scan_shape_name(i, buf, 128))
            out[buf.value.decode()] = round(float(ms[i]), 4)
        return out

    def reset_timings(self):
        n = C.c_uint64()
        self._check(lib().bmg_reset_timings(self.h, C.byref(n)))
        return n.value

    def finish(self):
        self._check(lib().bmg_finish(self.h))


def precompute_noalloc(d_packed, n, p, recode, types, d_out, d_flag, stream=None):
    """bmg_precompute_noalloc on caller-owned device buffers (raw pointers)."""
    t = (C.c_int32 * len(types))(*types)
    off = C.c_uint32()
    rc = lib().bmg_precompute_noalloc(C.c_void_p(d_packed), n, p, int(recode), t, len(types),
                                      C.c_void_p(d_out), C.byref(off), C.c_void_p(d_flag),
                                      None if stream is None else C.c_void_p(stream))
    if rc != 0:
        raise BmgError(rc, "bmg_precompute_noalloc failed")
    return off.value


def scan_shapes():
    """Descriptions of the tensor-core scan's launch shapes, in shape order."""
    out = []
    buf = C.create_string_buffer(128)
    while lib().bmg_get_scan_shape_name(len(out), buf, 128) == 0:
        out.append(buf.value.decode())
    return out


def selftest_exp(a):
    """The scan's table-driven exp of each |a| <= 700 (bmg_selftest_exp)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    out = np.empty_like(a)
    rc = lib().bmg_selftest_exp(_ptr(a), _ptr(out), a.size)
    if rc != 0:
        raise BmgError(rc, "bmg_selftest_exp failed")
    return out


def run_ini(path, n_iter=None, write_files=True):
    """Run a reference INI end to end on the GPU, writing the reference's files."""
    opt = options_from_ini(path, quiet=False)
    opt.write_files = 1 if write_files else 0
    packed, y, e = read_plink(opt)
    ctx = Context(opt)
    ctx.load_bed(packed)
    ctx.set_phenotypes(y)
    ctx.set_covariates(e)
    ctx.precompute()
    ctx.run(opt.do_n_iter if n_iter is None else n_iter, collect=False)
    ctx.finish()
    return ctx
