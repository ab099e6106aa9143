"""Python access to the GB300 population evaluator (libppi_gpu.so).

Everything here goes through the C ABI of include/ppi_gpu.h with ctypes; the
compute runs only in the CUDA kernels of that library.  If the library is not
built, importing the binding raises: there is no CPU fallback.
"""
from .grammar import Grammar, load as load_grammar, parse_bnf  # noqa: F401
from ._lib import (Evaluator, BatchEvaluator, BATCH_GRAPH, BATCH_AUTOTUNE, PpiGpuError, STRATEGY, ERROR_FN, MATH,  # noqa: F401
                   exported_symbols, lib_path, load_library, read_csv)
