"""The C-ABI library loads and exports every entry point include/ppi_gpu.h
declares (no GPU needed: nothing here launches work)."""
import ctypes
import os
import subprocess

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
    assert lib.ppi_gpu_version().decode() == "ppi_gpu 1 sm_103a"


def test_invalid_config_is_rejected_without_device(lib):
    cfg = ppi_gpu._lib.Config()
    h = ctypes.c_void_p()
    assert lib.ppi_gpu_create(ctypes.byref(cfg), ctypes.byref(h)) == 1   # max_size 0
    assert lib.ppi_gpu_create(None, ctypes.byref(h)) == 1


def test_library_contains_only_sm_103a_code():
    out = subprocess.run(["cuobjdump", "--list-elf", B.LIB], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    arches = {l.split(".")[-2] for l in out.stdout.split() if l.endswith(".cubin")}
    assert arches == {"sm_103a"}, arches
