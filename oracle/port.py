"""Python handle on the CPU oracle (oracle/port) and on the reference build.

ORACLE / TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg, as the oracle.  The product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from bmagwa_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libbmgport.so")
REF_BIN = os.path.join(HERE, "_ref", "bmagwa_ref")
REF_PROBE = os.path.join(HERE, "_ref", "ref_probe")

_lib = None


def build(verbose=False):
    """Compile the port (and nothing else) into oracle/_build."""
    os.makedirs(os.path.dirname(PORT_LIB), exist_ok=True)
    inc = os.path.join(HERE, "..", "include")
    # no FMA contraction: the same arithmetic on x86-64 and aarch64 (gcc
    # contracts a*b+c by default where the target has FMA)
    cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-I" + inc,
           "-I" + os.path.join(HERE, "port"), os.path.join(HERE, "port", "port.cpp"),
           "-x", "c", os.path.join(HERE, "linalg.c"), "-o", PORT_LIB, "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    return PORT_LIB


def reference_dir():
    """Where the reference tree is: $BMAGWA_REFERENCE, else the REF default of
    oracle/Makefile (the recipe that compiles it)."""
    env = os.environ.get("BMAGWA_REFERENCE")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REF ?="):
                return line.split("=", 1)[1].strip()
    return ""


def build_reference():
    """Compile the reference sources (needs the reference tree) into oracle/_ref."""
    subprocess.run(["make", "-s", "-C", HERE, "-j8", "REF=" + reference_dir()], check=True)
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(HERE, "port", "port.cpp"), os.path.join(HERE, "port", "port.h"),
                os.path.join(HERE, "linalg.c"), os.path.join(HERE, "..", "include", "bmg_rng.h"),
                os.path.join(HERE, "..", "include", "bmg.h")]
        if not os.path.exists(PORT_LIB) or any(os.path.getmtime(s) > os.path.getmtime(PORT_LIB)
                                               for s in srcs):
            build()
        L = C.CDLL(PORT_LIB)
        L.bmgport_create.argtypes = [C.POINTER(abi.Options), C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]
        L.bmgport_run.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(abi.TraceSink)]
        L.bmgport_scan.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        L.bmgport_scan_logodds.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
        L.bmgport_schur.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        L.bmgport_scan_yhat.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_double, C.c_void_p,
                                        C.c_void_p]
        L.bmgport_scan_yhat_logodds.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_double, C.c_void_p]
        L.bmgport_get_state.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(abi.ChainState),
                                        C.c_void_p, C.c_void_p, C.c_uint32]
        L.bmgport_get_rao.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        L.bmgport_get_last_scan.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        L.bmgport_get_proposal.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
        L.bmgport_get_precomputed.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32)]
        L.bmgport_get_data_stats.argtypes = [C.c_void_p, C.c_void_p]
        L.bmgport_get_genotypes.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_void_p]
        L.bmgport_model_lml.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p]
        L.bmgport_exh_modelset.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_uint32, C.c_void_p, C.c_void_p]
        L.bmgport_get_inv_tau2_alpha2.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
        L.bmgport_exh_proposal_probs.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_double, C.c_double, C.c_uint64, C.c_uint64,
                                                 C.c_void_p, C.c_void_p]
        L.bmgport_model_lml_remove.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_uint32, C.POINTER(C.c_double)]
        L.bmgport_dd_exercise.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_uint32,
                                          C.c_uint64, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
        L.bmgport_missing_step.argtypes = [C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
        L.bmgport_sample_beta_sigma2.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                                 C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint32,
                                                 C.POINTER(C.c_uint32)]
        L.bmgport_prior_terms.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]
        L.bmgport_destroy.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Port:
    """One oracle instance: all chains of an options struct on one dataset."""

    def __init__(self, opt, packed, y, e=None):
        self._keep = (np.ascontiguousarray(packed, dtype=np.uint8),
                      np.ascontiguousarray(y, dtype=np.float64),
                      None if e is None else np.ascontiguousarray(e, dtype=np.float64))
        self.opt = opt
        self.m_g = int(opt.m_g)
        self.n_types = int(opt.n_types)
        terms = set()
        for i in range(self.n_types):
            t = int(opt.types[i])
            terms.update((0, 1) if t == 4 else (t,))
        self.n_terms = len(terms)
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = lib().bmgport_create(C.byref(opt), _ptr(self._keep[0]), _ptr(self._keep[1]),
                                  _ptr(self._keep[2]), C.byref(h), err, 512)
        if rc != 0:
            raise RuntimeError("oracle: " + err.value.decode())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().bmgport_destroy(self.h)
            self.h = None

    def run(self, n_iter, threads=1):
        col = abi.TraceCollector()
        rc = lib().bmgport_run(self.h, n_iter, threads, C.byref(col.sink))
        if rc != 0:
            raise RuntimeError("oracle run failed")
        return col

    def scan(self, chain=0):
        pr = np.zeros(self.m_g)
        prt = np.zeros(self.m_g * self.n_types) if self.n_types > 1 else None
        if lib().bmgport_scan(self.h, chain, _ptr(pr), _ptr(prt)) != 0:
            raise RuntimeError("oracle scan failed")
        return pr, (prt.reshape(self.m_g, self.n_types) if prt is not None else None)

    def scan_logodds(self, chain=0):
        """Per-SNP log posterior odds of inclusion from an RB scan of the
        chain's current state."""
        lo = np.zeros(self.m_g)
        if lib().bmgport_scan_logodds(self.h, chain, _ptr(lo)) != 0:
            raise RuntimeError("oracle scan failed")
        return lo

    def schur(self, chain=0):
        """(p, terms) change of the model LML from adding each single term of
        each SNP outside the model (NaN inside), and the 4 prior precisions."""
        nt = self.n_terms
        out = np.zeros(self.m_g * nt)
        itv = np.zeros(4)
        if lib().bmgport_schur(self.h, chain, _ptr(out), _ptr(itv)) != 0:
            raise RuntimeError("oracle Schur scan failed")
        return out.reshape(self.m_g, nt), itv

    def scan_yhat(self, y_hat, sigma2, chain=0):
        pr = np.zeros(self.m_g)
        prt = np.zeros(self.m_g * self.n_types) if self.n_types > 1 else None
        yh = np.ascontiguousarray(y_hat, dtype=np.float64)
        if lib().bmgport_scan_yhat(self.h, chain, _ptr(yh), float(sigma2), _ptr(pr), _ptr(prt)) != 0:
            raise RuntimeError("oracle scan failed")
        return pr, (prt.reshape(self.m_g, self.n_types) if prt is not None else None)

    def scan_yhat_logodds(self, y_hat, sigma2, chain=0):
        """Per-SNP log posterior odds of the RB scan against y_hat and sigma2."""
        lo = np.zeros(self.m_g)
        yh = np.ascontiguousarray(y_hat, dtype=np.float64)
        if lib().bmgport_scan_yhat_logodds(self.h, chain, _ptr(yh), float(sigma2), _ptr(lo)) != 0:
            raise RuntimeError("oracle scan failed")
        return lo

    def state(self, chain=0, cap=4096):
        st = abi.ChainState()
        loci = np.zeros(cap, dtype=np.uint32)
        types = np.zeros(cap, dtype=np.uint8)
        lib().bmgport_get_state(self.h, chain, C.byref(st), _ptr(loci), _ptr(types), cap)
        k = st.model_size
        return st, loci[:k].copy(), types[:k].copy()

    def missing_step(self, snp, n_reps=1, chain=0):
        """n_reps imputations of a SNP's missing calls: (counts of the value
        imputed for its first missing call, corrected precomputed row, the
        four codings A, H, D, R after the last draw)."""
        off = self.precomputed().shape[1]
        xx = np.zeros(off)
        g = np.zeros((4, int(self.opt.n)))
        counts = np.zeros(3, dtype=np.uint64)
        rc = lib().bmgport_missing_step(self.h, chain, snp, n_reps, _ptr(xx), _ptr(g), _ptr(counts))
        if rc != 0:
            raise ValueError("bad argument")
        return counts, xx, g

    def sample_beta_sigma2(self, snps, t_inds, inv_pairs, n_samples, seed=1234):
        """(sigma2 draws, beta draws n_samples x blen) given the model of the
        listed terms, from a stream seeded with seed."""
        snps = np.ascontiguousarray(snps, dtype=np.uint32)
        t_inds = np.ascontiguousarray(t_inds, dtype=np.uint8)
        inv = np.ascontiguousarray(inv_pairs, dtype=np.float64).reshape(-1)
        cap = 1 + 2 * len(snps) + int(self.opt.m_e)
        s2 = np.zeros(n_samples)
        beta = np.zeros((n_samples, cap))
        blen = C.c_uint32()
        if lib().bmgport_sample_beta_sigma2(self.h, len(snps), _ptr(snps) if len(snps) else None,
                                            _ptr(t_inds) if len(snps) else None, _ptr(inv) if len(snps) else None,
                                            seed, n_samples, _ptr(s2), _ptr(beta), cap, C.byref(blen)) != 0:
            raise RuntimeError("oracle sampling failed")
        return s2, beta[:, :blen.value]

    def prior_terms(self, Ns, nl, ta, tr=0):
        """(log model prior of Ns, change on add of type ta with nl loci,
        change on removal of type ta with nl loci, change on switch ta -> tr)."""
        ns = np.ascontiguousarray(Ns, dtype=np.int32)
        out = np.zeros(4)
        if lib().bmgport_prior_terms(self.h, _ptr(ns), nl, ta, tr, _ptr(out)) != 0:
            raise ValueError("bad type")
        return out

    def inv_tau2_alpha2(self, chain=0):
        out = np.zeros(4)
        if lib().bmgport_get_inv_tau2_alpha2(self.h, chain, _ptr(out)) != 0:
            raise IndexError(chain)
        return out

    def rao(self, chain=0):
        p = np.zeros(self.m_g)
        pt = np.zeros(self.m_g * self.n_types) if self.n_types > 1 else None
        lib().bmgport_get_rao(self.h, chain, _ptr(p), _ptr(pt))
        return p, (pt.reshape(self.m_g, self.n_types) if pt is not None else None)

    def last_scan(self, chain=0):
        p = np.zeros(self.m_g)
        pt = np.zeros(self.m_g * self.n_types) if self.n_types > 1 else None
        lib().bmgport_get_last_scan(self.h, chain, _ptr(p), _ptr(pt))
        return p, (pt.reshape(self.m_g, self.n_types) if pt is not None else None)

    def proposal(self, chain=0):
        p = np.zeros(self.m_g)
        pt = np.zeros(self.m_g * self.n_types) if self.n_types > 1 else None
        lib().bmgport_get_proposal(self.h, chain, _ptr(p), _ptr(pt))
        return p, (pt.reshape(self.m_g, self.n_types) if pt is not None else None)

    def precomputed(self):
        off = C.c_uint32()
        lib().bmgport_get_precomputed(self.h, None, C.byref(off))
        xx = np.zeros(self.m_g * off.value)
        lib().bmgport_get_precomputed(self.h, _ptr(xx), C.byref(off))
        return xx.reshape(self.m_g, off.value)

    def data_stats(self):
        out = np.zeros(4)
        lib().bmgport_get_data_stats(self.h, _ptr(out))
        return out

    def genotypes(self, typ, snp):
        out = np.zeros(int(self.opt.n))
        if lib().bmgport_get_genotypes(self.h, typ, snp, _ptr(out)) != 0:
            raise IndexError(snp)
        return out

    def model_lml(self, snps, t_inds, inv_pairs):
        snps = np.ascontiguousarray(snps, dtype=np.uint32)
        t_inds = np.ascontiguousarray(t_inds, dtype=np.uint8)
        inv = np.ascontiguousarray(inv_pairs, dtype=np.float64).reshape(-1)
        out = np.zeros(len(snps))
        if lib().bmgport_model_lml(self.h, len(snps), _ptr(snps), _ptr(t_inds), _ptr(inv),
                                   _ptr(out)) != 0:
            raise RuntimeError("oracle model failed")
        return out

    def model_lml_remove(self, snps, t_inds, inv_pairs, rem):
        """LML after adding the terms in order and removing model index rem."""
        snps = np.ascontiguousarray(snps, dtype=np.uint32)
        t_inds = np.ascontiguousarray(t_inds, dtype=np.uint8)
        inv = np.ascontiguousarray(inv_pairs, dtype=np.float64).reshape(-1)
        out = C.c_double()
        if lib().bmgport_model_lml_remove(self.h, len(snps), _ptr(snps), _ptr(t_inds), _ptr(inv), rem,
                                          C.byref(out)) != 0:
            raise RuntimeError("oracle model failed")
        return out.value

    def exh_modelset(self, snps, t_inds, inv_pairs, const_loci):
        """(exhaustive, direct): log probabilities of the 2^m sub-models of the
        last m = len(snps) - const_loci terms, by the delayed-rejection
        enumeration and by building each model from scratch."""
        snps = np.ascontiguousarray(snps, dtype=np.uint32)
        t_inds = np.ascontiguousarray(t_inds, dtype=np.uint8)
        inv = np.ascontiguousarray(inv_pairs, dtype=np.float64).reshape(-1)
        nm = len(snps) - const_loci
        exh, direct = np.zeros(1 << nm), np.zeros(1 << nm)
        if lib().bmgport_exh_modelset(self.h, len(snps), _ptr(snps), _ptr(t_inds), _ptr(inv),
                                      const_loci, _ptr(exh), _ptr(direct)) != 0:
            raise RuntimeError("oracle exhaustive model set failed")
        return exh, direct


def exh_proposal_probs(bit_to_order, q_add, q_rem, z_add, z_rem, const_loci, m_g, log_q_add_types=None):
    """Log proposal probabilities of the 2^m sub-models of a delayed-rejection
    move (src/sampler.cpp:980-1049), m = len(q_add), in bit order."""
    m = len(q_add)
    order = np.ascontiguousarray(bit_to_order, dtype=np.uint8)
    qa = np.ascontiguousarray(q_add, dtype=np.float64)
    qr = np.ascontiguousarray(q_rem, dtype=np.float64)
    lt = None if log_q_add_types is None else np.ascontiguousarray(log_q_add_types, dtype=np.float64)
    out = np.zeros(1 << m)
    if lib().bmgport_exh_proposal_probs(int(lt is not None), m, _ptr(order), _ptr(qa), _ptr(qr), z_add, z_rem,
                                        const_loci, m_g, None if lt is None else _ptr(lt), _ptr(out)) != 0:
        raise ValueError("move size out of range")
    return out


def dd_exercise(w, ops=(), seed=1234, n_samples=0):
    """The proposal tree alone (src/discrete_distribution.hpp:64-330): apply
    ops (k >= 0 zeroes SNP k, k < 0 restores SNP -k - 1); returns (node values,
    total weight, draw counts per SNP)."""
    w = np.ascontiguousarray(w, dtype=np.float64)
    o = np.ascontiguousarray(ops, dtype=np.int64)
    vals = np.zeros(len(w))
    counts = np.zeros(len(w), dtype=np.uint64)
    tot = C.c_double()
    rc = lib().bmgport_dd_exercise(_ptr(w), len(w), _ptr(o) if len(o) else None, len(o), seed, n_samples,
                                   _ptr(vals), C.byref(tot), _ptr(counts))
    if rc != 0:
        raise ValueError("dd_exercise failed (%d)" % rc)
    return vals, tot.value, counts


def read_ref_outputs(basename, chain, m_g, n_types=1):
    """Read the binary trace files the reference (or libbmg) writes for a chain."""
    b = "%s%d" % (basename, chain)
    rd = lambda suf, dt: np.fromfile(b + suf, dtype=dt) if os.path.exists(b + suf) else None
    out = {
        "jumpdistance": rd("_jumpdistance.dat", np.uint8),
        "move_type": rd("_move_type.dat", np.uint8),
        "move_size": rd("_move_size.dat", np.uint8),
        "modelsize": rd("_modelsize.dat", np.uint32),
        "loci": rd("_loci.dat", np.uint32),
        "log_likelihood": rd("_log_likelihood.dat", np.float64),
        "log_prior": rd("_log_prior.dat", np.float64),
        "sigma2": rd("_sigma2.dat", np.float64),
        "alpha": rd("_alpha.dat", np.float64),
        "pve": rd("_pve.dat", np.float64),
        "rao": rd("_rao.dat", np.float64),
        "types": rd("_types.dat", np.uint8),
        "rao_types": rd("_rao_types.dat", np.float64),
        "beta": rd("_beta.dat", np.float64),
    }
    return out
