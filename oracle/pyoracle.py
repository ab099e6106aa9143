"""ctypes access to the CPU oracle (libppi_oracle.so) and to the reference
builds in oracle/_ref/ (libref_seq / libref_cl / libref_decode).

TEST INFRASTRUCTURE: imported by tests/, __graft_entry__.smoke() and the CPU
legs of bench.py only.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "libppi_oracle.so")

EF = {"abs": 0, "squared": 1, "misclass": 2, "cost": 3}
STRATEGY = {"PP": 0, "SEQ": 0, "DP": 1, "PDP": 2}

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint8)


def build(quiet=True):
    """Compile the oracle restatement (gcc, OpenMP, no fused multiply-add)."""
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", os.path.join(HERE, "ppi_oracle.c"), "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True, capture_output=quiet)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class _Cfg(C.Structure):
    _fields_ = [("nlin", C.c_int), ("ncol", C.c_int), ("rows", _fp), ("error_fn", C.c_int),
                ("cost", _fp), ("cost_n", C.c_int), ("reduce_max", C.c_int),
                ("protected_fns", C.c_int), ("float_math", C.c_int), ("sym_values", _ip),
                ("sym_ops", _ip), ("sym_literals", _fp), ("n_syms", C.c_int), ("threads", C.c_int)]


def _f(a):
    return a.ctypes.data_as(_fp)


def _i(a):
    return a.ctypes.data_as(_ip)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.ppio_evaluate.argtypes = [C.POINTER(_Cfg), C.c_int, C.c_int, _ip, _fp, _ip, C.c_int,
                                    C.c_int, C.c_float, _fp]
        L.ppio_predict.argtypes = [C.POINTER(_Cfg), _ip, _fp, C.c_int, _fp]
        L.ppio_best_index.argtypes = [_fp, C.c_int]
        L.ppio_best_index_accelerator.argtypes = [_fp, C.c_int, C.c_int]
        L.ppio_evaluate64.argtypes = [C.POINTER(_Cfg), _ip, _fp, _ip, C.c_int, C.c_int, C.c_double,
                                      C.POINTER(C.c_double)]
        _dp = C.POINTER(C.c_double)
        L.ppio_adjoint64.argtypes = [C.POINTER(_Cfg), _ip, _dp, _ip, C.c_int, C.c_int, C.c_int, _dp,
                                     _dp]
        L.ppio_decode.argtypes = [_ip, _ip, _ip, _ip, C.c_int, C.c_int, C.c_int, _up, C.c_int,
                                  C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, _ip,
                                  _fp, _ip]
        _lib = L
    return _lib


class Oracle:
    """Runtime-configured CPU oracle over one dataset."""

    def __init__(self, rows, symtab, error_fn="abs", cost=None, reduce_max=False,
                 protected=False, float_math=False, threads=0):
        self.rows = np.ascontiguousarray(rows, np.float32)
        self.nlin, self.ncol = self.rows.shape
        self.sv, self.so, self.sl = [np.ascontiguousarray(a) for a in symtab]
        self.cost = None if cost is None else np.ascontiguousarray(cost, np.float32)
        self.cfg = _Cfg(self.nlin, self.ncol, _f(self.rows), EF[error_fn],
                        _f(self.cost) if self.cost is not None else None,
                        0 if self.cost is None else self.cost.shape[0], int(reduce_max),
                        int(protected), int(float_math), _i(self.sv), _i(self.so), _f(self.sl),
                        len(self.sv), threads)

    def evaluate(self, phenotype, ephemeral, size, strategy="PP", lanes=1, alpha=0.0):
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        sz = np.ascontiguousarray(size, np.int32)
        n, mps = ph.shape
        out = np.empty(n, np.float32)
        rc = lib().ppio_evaluate(C.byref(self.cfg), STRATEGY[strategy], lanes, _i(ph), _f(ep),
                                 _i(sz), mps, n, alpha, _f(out))
        assert rc == 0
        return out

    def evaluate64(self, phenotype, ephemeral, size, alpha=0.0):
        """FP64 re-evaluation (ppio_evaluate64): double fitness, HUGE_VAL
        (inf) where the float evaluators give the FLT_MAX sentinel's cases."""
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        sz = np.ascontiguousarray(size, np.int32)
        n, mps = ph.shape
        out = np.empty(n, np.float64)
        assert lib().ppio_evaluate64(C.byref(self.cfg), _i(ph), _f(ep), _i(sz), mps, n, alpha,
                                     out.ctypes.data_as(C.POINTER(C.c_double))) == 0
        return out

    def adjoint64(self, phenotype, ephemeral, size, float_forward=False):
        """FP64 fitness and d(fitness)/d(ephemeral) (ppio_adjoint64); ephemeral
        is taken in double so a finite-difference caller can perturb it finely.
        float_forward: node values in the reference's float semantics."""
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float64)
        sz = np.ascontiguousarray(size, np.int32)
        n, mps = ph.shape
        fit = np.empty(n, np.float64)
        grad = np.empty((n, mps), np.float64)
        dp = C.POINTER(C.c_double)
        assert lib().ppio_adjoint64(C.byref(self.cfg), _i(ph), ep.ctypes.data_as(dp), _i(sz), mps, n,
                                    int(float_forward), fit.ctypes.data_as(dp),
                                    grad.ctypes.data_as(dp)) == 0
        return fit, grad

    def predict(self, phenotype, ephemeral, size):
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        out = np.empty(self.nlin, np.float32)
        assert lib().ppio_predict(C.byref(self.cfg), _i(ph), _f(ep), int(size), _f(out)) == 0
        return out


def best_index(fitness):
    f = np.ascontiguousarray(fitness, np.float32)
    return lib().ppio_best_index(_f(f), len(f))


def best_index_accelerator(values, group):
    """acc_interpret's best index: best_individual over work-groups of
    `group` values, then PickNBest over the group winners."""
    v = np.ascontiguousarray(values, np.float32)
    return lib().ppio_best_index_accelerator(_f(v), len(v), int(group))


def decode(grammar, genomes, bits_per_gene, bits_per_constant, lo, hi, max_size):
    first, count, alen, asyms = grammar.decode_tables()
    g = np.ascontiguousarray(genomes, np.uint8)
    n, nb = g.shape
    ph = np.zeros((n, max_size), np.int32)
    ep = np.zeros((n, max_size), np.float32)
    sz = np.zeros(n, np.int32)
    tc = grammar.t_const if grammar.t_const is not None else -1
    ta = grammar.t_attribute if grammar.t_attribute is not None else -1
    lib().ppio_decode(_i(first), _i(count), _i(alen), _i(np.ascontiguousarray(asyms)),
                      grammar.max_rule, tc, ta, g.ctypes.data_as(_up), n, nb, bits_per_gene,
                      bits_per_constant, lo, hi, max_size, _i(ph), _f(ep), _i(sz))
    return ph, ep, sz


# ---- reference builds (oracle/_ref, present only where the reference was built) ----

def ref_csv_read(path):
    """The reference's own read() (src/main.cc:32-119): (status, array or
    None).  Its messages go to stderr, as in PPI.  None when oracle/_ref has
    no CSV build."""
    so = os.path.join(REF, "libref_csv.so")
    if not os.path.exists(so):
        return None
    L = C.CDLL(so)
    L.ref_csv_read.argtypes = [C.c_char_p, _fp, C.c_long, _ip, _ip]
    nlin = np.zeros(1, np.int32)
    ncol = np.zeros(1, np.int32)
    rc = L.ref_csv_read(os.fsencode(path), None, 0, _i(nlin), _i(ncol))
    if rc != 0:
        return rc, None
    out = np.zeros((int(nlin[0]), int(ncol[0])), np.float32)
    rc = L.ref_csv_read(os.fsencode(path), _f(out), out.size, _i(nlin), _i(ncol))
    return rc, out


def ref_manifest():
    p = os.path.join(REF, "manifest.json")
    return json.load(open(p)) if os.path.exists(p) else {}


class RefBuild:
    """One reference configuration compiled by oracle/build_ref.py."""

    def __init__(self, name):
        self.name = name
        self.info = ref_manifest()[name]
        d = os.path.join(REF, name)
        self.seq = C.CDLL(os.path.join(d, "libref_seq.so"))
        self.cl = C.CDLL(os.path.join(d, "libref_cl.so"))
        self.dec = C.CDLL(os.path.join(d, "libref_decode.so"))
        self.seq.ref_seq_init.argtypes = [C.c_uint, _fp, C.c_int, C.c_int]
        self.seq.ref_seq_interpret.argtypes = [_ip, _fp, _ip, _fp, C.c_int, _ip, C.c_int, C.c_int,
                                               C.c_int, C.c_float]
        self.cl.ref_cl_evaluate.argtypes = [C.c_int, _ip, _fp, _ip, _fp, C.c_int, C.c_int,
                                            C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, _fp,
                                            _ip]
        self.dec.ref_decode.argtypes = [_up, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float,
                                        C.c_float, C.c_uint, C.c_int, _ip, _fp, _ip, _ip]
        self.max_size = self.cl.ref_cl_max_phenotype_size()

    def seq_evaluate(self, rows, phenotype, ephemeral, size, alpha=0.0, prediction=False):
        rows = np.ascontiguousarray(rows, np.float32)
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        sz = np.ascontiguousarray(size, np.int32)
        n, mps = ph.shape
        self.seq.ref_seq_init(mps, _f(rows), rows.shape[0], rows.shape[1])
        out = np.empty(rows.shape[0] if prediction else n, np.float32)
        idx = np.zeros(1, np.int32)
        self.seq.ref_seq_interpret(_i(ph), _f(ep), _i(sz), _f(out), n, _i(idx), 1,
                                   1 if prediction else 0, 1 if prediction else 0, alpha)
        self.seq.ref_seq_destroy()
        return out, int(idx[0])

    def cl_evaluate(self, strategy, rows, phenotype, ephemeral, size, local1, local2=64,
                    alpha=0.0, prediction=False):
        rows = np.ascontiguousarray(rows, np.float32)
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        sz = np.ascontiguousarray(size, np.int32)
        n, mps = ph.shape
        assert mps == self.max_size, "programs must use the build's MAX_PHENOTYPE_SIZE"
        out = np.empty(rows.shape[0] if prediction else n, np.float32)
        idx = np.zeros(1, np.int32)
        rc = self.cl.ref_cl_evaluate(STRATEGY[strategy], _i(ph), _f(ep), _i(sz), _f(rows),
                                     rows.shape[0], rows.shape[1], n, int(prediction), local1,
                                     local2, alpha, _f(out), None if prediction else _i(idx))
        assert rc == 0
        return out, int(idx[0])

    def decode(self, genomes, bits_per_gene, bits_per_constant, lo, hi, max_size, slack=16):
        g = np.ascontiguousarray(genomes, np.uint8)
        n, nb = g.shape
        stride = max_size + slack
        ph = np.zeros((n, stride), np.int32)
        ep = np.zeros((n, stride), np.float32)
        sz = np.zeros(n, np.int32)
        al = np.zeros(n, np.int32)
        self.dec.ref_decode(g.ctypes.data_as(_up), n, nb, bits_per_gene, bits_per_constant, lo,
                            hi, max_size, stride, _i(ph), _f(ep), _i(sz), _i(al))
        return ph, ep, sz, al
