"""ctypes binding of include/ppi_gpu.h.

``Evaluator`` mirrors the reference's interpreter interface
(src/interpreter/accelerator.h): construct with the run configuration
(acc_interpret_init), ``set_dataset`` (the one dataset upload), ``evaluate``
one generation (acc_interpret with ppp_mode = 0), ``predict`` one program
(ppp prediction mode).  Errors raise ``PpiGpuError`` carrying the C status.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

from . import build as _build

STRATEGY = {"PP": 0, "DP": 1, "PDP": 2}
ERROR_FN = {"abs": 0, "squared": 1, "misclass": 2, "cost": 3}
MATH = {"fast": 0, "parity": 1, "native": 2}
STATUS = {0: "PPI_OK", 1: "PPI_ERR_INVALID_ARGUMENT", 2: "PPI_ERR_CUDA",
          3: "PPI_ERR_OUT_OF_MEMORY", 4: "PPI_ERR_UNSUPPORTED", 5: "PPI_ERR_NOT_READY",
          6: "PPI_ERR_DEVICE_STATUS"}

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_up = C.POINTER(C.c_uint8)


class PpiGpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, status), message))
        self.status = status


class SymbolEntry(C.Structure):
    _fields_ = [("symbol", C.c_int32), ("op", C.c_int32), ("value", C.c_float)]


class Config(C.Structure):
    _fields_ = [("max_size", C.c_int32), ("population_size", C.c_int32), ("strategy", C.c_int32),
                ("lanes", C.c_int32), ("error_fn", C.c_int32), ("reduce_max", C.c_int32),
                ("protected_fns", C.c_int32), ("math", C.c_int32), ("cost", _fp),
                ("cost_n", C.c_int32), ("symbols", C.POINTER(SymbolEntry)),
                ("n_symbols", C.c_int32), ("device", C.c_int32), ("best_rule", C.c_int32),
                ("best_group", C.c_int32)]


# ppi_best_rule: "accelerator" = the index acc_interpret returns (best_individual
# work-groups + PickNBest), "sequential" = the index seq_interpret returns.
BEST_RULE = {"accelerator": 0, "sequential": 1}


class BatchPopulation(C.Structure):
    _fields_ = [("rows", _fp), ("nlin", C.c_int32), ("ncol", C.c_int32), ("n", C.c_int32),
                ("strategy", C.c_int32), ("lanes", C.c_int32), ("error_fn", C.c_int32),
                ("reduce_max", C.c_int32), ("protected_fns", C.c_int32), ("cost", _fp),
                ("cost_n", C.c_int32)]


BATCH_GRAPH = 1
BATCH_AUTOTUNE = 2


def lib_path():
    return _build.LIB


_lib = None


def load_library():
    """Load libppi_gpu.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError("libppi_gpu.so is not built (%s); run __graft_entry__.build()" % path)
    L = C.CDLL(path)
    L.ppi_gpu_version.restype = C.c_char_p
    L.ppi_gpu_last_error.restype = C.c_char_p
    L.ppi_gpu_last_error.argtypes = [C.c_void_p]
    L.ppi_gpu_create.argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
    L.ppi_gpu_destroy.argtypes = [C.c_void_p]
    L.ppi_gpu_set_dataset_rowmajor.argtypes = [C.c_void_p, _fp, C.c_int32, C.c_int32]
    L.ppi_gpu_set_dataset.argtypes = [C.c_void_p, C.POINTER(_fp), C.c_int32, C.c_int32]
    L.ppi_gpu_evaluate.argtypes = [C.c_void_p, _ip, _fp, _ip, C.c_int32, C.c_float, _fp, _ip]
    L.ppi_gpu_evaluate_launch.argtypes = L.ppi_gpu_evaluate.argtypes
    L.ppi_gpu_evaluate_wait.argtypes = [C.c_void_p]
    L.ppi_gpu_evaluate_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_int32, C.c_float, C.c_void_p, C.c_void_p,
                                          C.c_void_p]
    L.ppi_gpu_predict.argtypes = [C.c_void_p, _ip, _fp, C.c_int32, _fp]
    L.ppi_gpu_set_grammar.argtypes = [C.c_void_p, _ip, _ip, C.c_int32, _ip, _ip, C.c_int32,
                                      C.c_int32, C.c_int32, C.c_int32]
    L.ppi_gpu_decode.argtypes = [C.c_void_p, _up, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                 C.c_float, C.c_float, _ip, _fp, _ip]
    L.ppi_gpu_decode_evaluate.argtypes = [C.c_void_p, _up, C.c_int32, C.c_int32, C.c_int32,
                                          C.c_int32, C.c_float, C.c_float, C.c_float, _fp, _ip,
                                          _ip]
    L.ppi_gpu_last_kernel_ms.argtypes = [C.c_void_p, _fp]
    L.ppi_gpu_last_launch_count.argtypes = [C.c_void_p]
    L.ppi_gpu_last_stage_ms.argtypes = [C.c_void_p, _fp, _fp]
    L.ppi_gpu_lanes.argtypes = [C.c_void_p]
    L.ppi_gpu_translation.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_uint32), _ip, _ip, _ip]
    L.ppi_gpu_set_dataset_csv.argtypes = [C.c_void_p, C.c_char_p, _ip, _ip]
    L.ppi_csv_read.argtypes = [C.c_char_p, _fp, C.c_int64, C.c_int32, _ip, _ip, C.c_char_p,
                               C.c_int32]
    L.ppi_gpu_kernel_arch.restype = C.c_int32
    L.ppi_gpu_constant_gradient.argtypes = [C.c_void_p, _ip, _fp, _ip, C.c_int32, _fp]
    L.ppi_batch_create.argtypes = [C.POINTER(Config), C.c_int32, C.POINTER(BatchPopulation),
                                   C.POINTER(C.c_void_p)]
    L.ppi_batch_destroy.argtypes = [C.c_void_p]
    L.ppi_batch_last_error.restype = C.c_char_p
    L.ppi_batch_last_error.argtypes = [C.c_void_p]
    L.ppi_batch_set_alpha.argtypes = [C.c_void_p, _fp]
    L.ppi_batch_evaluate.argtypes = [C.c_void_p, _ip, _fp, _ip, _fp, _ip, C.c_int32]
    L.ppi_batch_evaluate_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
    L.ppi_batch_last_kernel_ms.argtypes = [C.c_void_p, _fp]
    L.ppi_batch_shape.argtypes = [C.c_void_p, _ip, _ip, _ip, _fp]
    L.ppi_batch_set_shape.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    L.ppi_batch_last_launch_count.argtypes = [C.c_void_p, _ip]
    _lib = L
    return L


def exported_symbols(header=None):
    """Function names declared in include/ppi_gpu.h (for export checks)."""
    header = header or os.path.join(_build.INCLUDE, "ppi_gpu.h")
    text = open(header).read()
    return sorted(set(re.findall(r"\b(ppi_(?:gpu|batch|csv)_\w+)\s*\(", text)))


def read_csv(path):
    """PPI's training CSV read by the library's reader (ppi_csv_read, the
    rules of src/main.cc:32-122): a row-major nlin x ncol float32 array;
    raises PpiGpuError with the reader's message for a file it rejects."""
    L = load_library()
    nlin = np.zeros(1, np.int32)
    ncol = np.zeros(1, np.int32)
    msg = C.create_string_buffer(512)
    p = os.fsencode(path)
    st = L.ppi_csv_read(p, None, 0, 0, _i(nlin), _i(ncol), msg, 512)
    if st != 0:
        raise PpiGpuError(st, msg.value.decode())
    cm = np.zeros((int(ncol[0]), max(1, int(nlin[0]))), np.float32)
    st = L.ppi_csv_read(p, _f(cm), cm.size, cm.shape[1], _i(nlin), _i(ncol), msg, 512)
    if st != 0:
        raise PpiGpuError(st, msg.value.decode())
    return np.ascontiguousarray(cm[:, :int(nlin[0])].T)


def _f(a):
    return a.ctypes.data_as(_fp)


def _i(a):
    return a.ctypes.data_as(_ip)


class Evaluator:
    """One evaluator instance on one GPU (a handle of the C ABI)."""

    def __init__(self, symtab, max_size, population_size, strategy="PDP", lanes=0,
                 error_fn="abs", cost=None, reduce_max=False, protected=False, math="fast",
                 device=0, best_rule="accelerator", best_group=0):
        L = load_library()
        sv, so, sl = symtab
        self._syms = (SymbolEntry * max(1, len(sv)))()
        for k in range(len(sv)):
            self._syms[k] = SymbolEntry(int(sv[k]), int(so[k]), float(sl[k]))
        self._cost = None if cost is None else np.ascontiguousarray(cost, np.float32)
        cfg = Config(max_size, population_size, STRATEGY[strategy], lanes, ERROR_FN[error_fn],
                     int(reduce_max), int(protected), MATH[math],
                     _f(self._cost) if self._cost is not None else None,
                     0 if self._cost is None else self._cost.shape[0], self._syms, len(sv),
                     device, BEST_RULE[best_rule], int(best_group))
        self._config = cfg
        h = C.c_void_p()
        st = L.ppi_gpu_create(C.byref(cfg), C.byref(h))
        if st != 0:
            raise PpiGpuError(st, "ppi_gpu_create failed")
        self._h = h
        self._L = L
        self.max_size = max_size
        self.population_size = population_size
        self.nlin = 0

    def _check(self, st):
        if st != 0:
            raise PpiGpuError(st, self._L.ppi_gpu_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.ppi_gpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_dataset(self, rows):
        self._rows = np.ascontiguousarray(rows, np.float32)
        nlin, ncol = self._rows.shape
        self._check(self._L.ppi_gpu_set_dataset_rowmajor(self._h, _f(self._rows), nlin, ncol))
        self.nlin = nlin

    def set_dataset_csv(self, path):
        """PPI's training CSV straight to the device (ppi_gpu_set_dataset_csv)."""
        nlin = np.zeros(1, np.int32)
        ncol = np.zeros(1, np.int32)
        self._check(self._L.ppi_gpu_set_dataset_csv(self._h, os.fsencode(path), _i(nlin), _i(ncol)))
        self.nlin = int(nlin[0])
        return int(nlin[0]), int(ncol[0])

    def evaluate(self, phenotype, ephemeral, size, alpha=0.0):
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        sz = np.ascontiguousarray(size, np.int32)
        n = len(sz)
        assert ph.shape == (n, self.max_size) and ep.shape == (n, self.max_size)
        fit = np.empty(n, np.float32)
        best = np.zeros(1, np.int32)
        self._check(self._L.ppi_gpu_evaluate(self._h, _i(ph), _f(ep), _i(sz), n, alpha, _f(fit),
                                             _i(best)))
        return fit, int(best[0])

    def evaluate_device(self, d_ph, d_eph, d_size, n, alpha, d_fit, d_best, stream=0):
        """Device pointers (ints) in, queued on `stream`; no synchronisation."""
        self._check(self._L.ppi_gpu_evaluate_device(self._h, d_ph, d_eph, d_size, n, alpha,
                                                    d_fit, d_best, stream))

    def constant_gradient(self, phenotype, ephemeral, size):
        """d(fitness)/d(ephemeral[i][k]) at every CONST token (0 elsewhere)."""
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        sz = np.ascontiguousarray(size, np.int32)
        n = len(sz)
        assert ph.shape == (n, self.max_size) and ep.shape == (n, self.max_size)
        grad = np.empty((n, self.max_size), np.float32)
        self._check(self._L.ppi_gpu_constant_gradient(self._h, _i(ph), _f(ep), _i(sz), n, _f(grad)))
        return grad

    def predict(self, phenotype, ephemeral, size):
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        out = np.empty(self.nlin, np.float32)
        self._check(self._L.ppi_gpu_predict(self._h, _i(ph), _f(ep), int(size), _f(out)))
        return out

    def set_grammar(self, grammar):
        first, count, alen, asyms = grammar.decode_tables()
        self._dec = (first, count, alen, np.ascontiguousarray(asyms))
        tc = grammar.t_const if grammar.t_const is not None else -1
        ta = grammar.t_attribute if grammar.t_attribute is not None else -1
        self._check(self._L.ppi_gpu_set_grammar(self._h, _i(first), _i(count), len(first),
                                                _i(alen), _i(self._dec[3]), len(alen),
                                                grammar.max_rule, tc, ta))

    def decode(self, genomes, bits_per_gene, bits_per_constant, lo, hi):
        g = np.ascontiguousarray(genomes, np.uint8)
        n, nb = g.shape
        ph = np.zeros((n, self.max_size), np.int32)
        ep = np.zeros((n, self.max_size), np.float32)
        sz = np.zeros(n, np.int32)
        self._check(self._L.ppi_gpu_decode(self._h, g.ctypes.data_as(_up), n, nb, bits_per_gene,
                                           bits_per_constant, lo, hi, _i(ph), _f(ep), _i(sz)))
        return ph, ep, sz

    def decode_evaluate(self, genomes, bits_per_gene, bits_per_constant, lo, hi, alpha=0.0):
        g = np.ascontiguousarray(genomes, np.uint8)
        n, nb = g.shape
        fit = np.empty(n, np.float32)
        best = np.zeros(1, np.int32)
        sz = np.zeros(n, np.int32)
        self._check(self._L.ppi_gpu_decode_evaluate(self._h, g.ctypes.data_as(_up), n, nb,
                                                    bits_per_gene, bits_per_constant, lo, hi,
                                                    alpha, _f(fit), _i(best), _i(sz)))
        return fit, int(best[0]), sz

    def last_kernel_ms(self):
        ms = np.zeros(1, np.float32)
        self._check(self._L.ppi_gpu_last_kernel_ms(self._h, _f(ms)))
        return float(ms[0])

    def last_stage_ms(self):
        t = np.zeros(2, np.float32)
        self._check(self._L.ppi_gpu_last_stage_ms(self._h, _f(t[0:1]), _f(t[1:2])))
        return float(t[0]), float(t[1])

    def translation(self, n):
        """The last evaluate call's bytecode: (code uint32 [n, stride, 2],
        meta int32 [n, 2], opset) -- see ppi_gpu_translation."""
        stride = np.zeros(1, np.int32)
        opset = np.zeros(1, np.int32)
        self._check(self._L.ppi_gpu_translation(self._h, 0, None, None, _i(stride), _i(opset)))
        code = np.zeros((n, int(stride[0]), 2), np.uint32)
        meta = np.zeros((n, 2), np.int32)
        self._check(self._L.ppi_gpu_translation(self._h, n, code.ctypes.data_as(C.POINTER(C.c_uint32)),
                                                _i(meta), _i(stride), _i(opset)))
        return code, meta, int(opset[0])

    @property
    def lanes(self):
        return int(self._L.ppi_gpu_lanes(self._h))

    def geometry(self):
        """(threads per CTA, main-pass tile rows, record chunks per program)."""
        b, r, c = (np.zeros(1, np.int32) for _ in range(3))
        self._check(self._L.ppi_gpu_geometry(self._h, _i(b), _i(r), _i(c)))
        return int(b[0]), int(r[0]), int(c[0])

    def last_launch_count(self):
        return int(self._L.ppi_gpu_last_launch_count(self._h))


class BatchEvaluator:
    """Many populations in one batched step (ppi_batch_* of the C ABI).

    pops: list of dicts with keys rows, n and optionally strategy, lanes,
    error_fn, cost, reduce_max, protected.  Programs, fitness: all
    populations concatenated in order (rows of max_size)."""

    def __init__(self, symtab, max_size, pops, math="fast", device=0, best_rule="accelerator",
                 best_group=0):
        L = load_library()
        sv, so, sl = symtab
        self._syms = (SymbolEntry * max(1, len(sv)))()
        for k in range(len(sv)):
            self._syms[k] = SymbolEntry(int(sv[k]), int(so[k]), float(sl[k]))
        cfg = Config(max_size, 1, 0, 0, 0, 0, 0, MATH[math], None, 0, self._syms, len(sv), device,
                     BEST_RULE[best_rule], int(best_group))
        self._keep = []
        arr = (BatchPopulation * len(pops))()
        for i, p in enumerate(pops):
            rows = np.ascontiguousarray(p["rows"], np.float32)
            cost = p.get("cost")
            cost = None if cost is None else np.ascontiguousarray(cost, np.float32)
            self._keep += [rows, cost]
            arr[i] = BatchPopulation(_f(rows), rows.shape[0], rows.shape[1], int(p["n"]),
                                     STRATEGY[p.get("strategy", "PDP")], int(p.get("lanes", 0)),
                                     ERROR_FN[p.get("error_fn", "abs")], int(p.get("reduce_max", 0)),
                                     int(p.get("protected", 0)),
                                     _f(cost) if cost is not None else None,
                                     0 if cost is None else cost.shape[0])
        h = C.c_void_p()
        st = L.ppi_batch_create(C.byref(cfg), len(pops), arr, C.byref(h))
        if st != 0:
            raise PpiGpuError(st, "ppi_batch_create failed")
        self._h, self._L = h, L
        self.max_size = max_size
        self.counts = [int(p["n"]) for p in pops]
        self.total = sum(self.counts)

    def _check(self, st):
        if st != 0:
            raise PpiGpuError(st, self._L.ppi_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.ppi_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_alpha(self, alpha):
        a = np.ascontiguousarray(alpha, np.float32)
        self._check(self._L.ppi_batch_set_alpha(self._h, _f(a)))

    def evaluate(self, phenotype, ephemeral, size, flags=0):
        ph = np.ascontiguousarray(phenotype, np.int32)
        ep = np.ascontiguousarray(ephemeral, np.float32)
        sz = np.ascontiguousarray(size, np.int32)
        assert ph.shape == (self.total, self.max_size)
        fit = np.empty(self.total, np.float32)
        best = np.zeros(len(self.counts), np.int32)
        self._check(self._L.ppi_batch_evaluate(self._h, _i(ph), _f(ep), _i(sz), _f(fit), _i(best),
                                               flags))
        return fit, best

    def evaluate_device(self, d_ph, d_eph, d_size, d_fit, d_best, stream=0, flags=0):
        self._check(self._L.ppi_batch_evaluate_device(self._h, d_ph, d_eph, d_size, d_fit, d_best,
                                                      stream, flags))

    def last_kernel_ms(self):
        ms = np.zeros(1, np.float32)
        self._check(self._L.ppi_batch_last_kernel_ms(self._h, _f(ms)))
        return float(ms[0])

    def shape(self):
        """(block, main-pass grid, (main rows, wide rows), autotuner timings)."""
        b = np.zeros(1, np.int32)
        g = np.zeros(1, np.int32)
        r = np.zeros(2, np.int32)
        t = np.zeros(2, np.float32)
        self._check(self._L.ppi_batch_shape(self._h, _i(b), _i(g), _i(r), _f(t)))
        return int(b[0]), int(g[0]), (int(r[0]), int(r[1])), (float(t[0]), float(t[1]))

    def last_launch_count(self):
        n = np.zeros(1, np.int32)
        self._check(self._L.ppi_batch_last_launch_count(self._h, _i(n)))
        return int(n[0])

    def set_shape(self, block, rows=0):
        self._check(self._L.ppi_batch_set_shape(self._h, block, rows))
