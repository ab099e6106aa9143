"""The C-ABI library loads and exports every entry point include/ppi_gpu.h
declares (no GPU needed: nothing here launches work)."""
import ctypes
import os

import pytest

import ppi_gpu
from ppi_gpu import build as B


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(B.LIB):
        B.build()
    return ppi_gpu.load_library()


def test_every_declared_function_is_exported(lib):
    names = ppi_gpu.exported_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_version_and_target(lib):
    assert lib.ppi_gpu_version().decode() == "ppi_gpu 2 sm_103a"


def test_invalid_config_is_rejected_without_device(lib):
    cfg = ppi_gpu._lib.Config()
    h = ctypes.c_void_p()
    assert lib.ppi_gpu_create(ctypes.byref(cfg), ctypes.byref(h)) == 1   # max_size 0
    assert lib.ppi_gpu_create(None, ctypes.byref(h)) == 1


def test_build_targets_only_sm_103a():
    """Every translation unit and the link get exactly one -gencode: sm_103a
    code, no PTX for other targets."""
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert not any("gencode" in f or "arch" in f for f in B.NVCC_FLAGS)


@pytest.mark.gpu
def test_kernels_run_as_sm_103a_binaries(lib):
    lib.ppi_gpu_kernel_arch.restype = ctypes.c_int32
    assert lib.ppi_gpu_kernel_arch() == 103


def _noalloc(lib):
    f = lib.ppi_gpu_evaluate_noalloc
    f.argtypes = [ctypes.POINTER(ppi_gpu._lib.Config), ctypes.c_void_p, ctypes.c_int32,
                  ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int32, ctypes.c_float, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _noalloc_config(symbols):
    arr = (ppi_gpu._lib.SymbolEntry * len(symbols))(*[ppi_gpu._lib.SymbolEntry(s, op, 0.0)
                                                      for s, op in symbols])
    cfg = ppi_gpu._lib.Config()
    cfg.max_size = 64
    cfg.population_size = 1
    cfg.symbols = arr
    cfg.n_symbols = len(symbols)
    return cfg, arr


def test_noalloc_size_checks_come_before_any_device_work(lib):
    """The no-alloc entry point rejects a symbol table whose range does not fit
    the dense lookup (computed in 64 bits: INT_MIN .. INT_MAX would overflow
    a 32-bit difference) and a batch beyond its fixed scratch, with
    PPI_ERR_UNSUPPORTED, before any CUDA call: the device pointers below are
    never touched and no GPU is needed."""
    f = _noalloc(lib)
    fake = 1 << 20   # aligned, never dereferenced
    args = lambda n: (fake, 10, 2, 12, fake, fake, fake, n, 0.0, fake, fake, None, None)
    wide, keep = _noalloc_config([(-2**31, 1), (2**31 - 1, 14)])
    assert f(ctypes.byref(wide), *args(4)) == 4
    wide2, keep2 = _noalloc_config([(0, 1), (1 << 22, 14)])      # 2^22 + 1 values
    assert f(ctypes.byref(wide2), *args(4)) == 4
    ok, keep3 = _noalloc_config([(10000, 1), (10001, 14)])
    assert f(ctypes.byref(ok), *args(200000)) == 4               # beyond the 64 MiB scratch
    bad_rule, keep4 = _noalloc_config([(10000, 1)])
    bad_rule.best_rule = 7
    assert f(ctypes.byref(bad_rule), *args(4)) == 1
