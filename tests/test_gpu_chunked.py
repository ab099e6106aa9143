"""Chunked evaluation: a PDP population (one lane per tile position) over a
dataset larger than L2 is evaluated as (program, record chunk) work items in
chunk-major order (programs in groups whose lane states fit in L2), the
lanes' partial sums carried between a program's chunks.  Each lane still
adds its records in record order, so the fitness must be bit-identical to
the unchunked evaluation (the batch path, which never chunks) and to the
oracle in parity math."""
import numpy as np
import pytest

from helpers import ProgramGen, assert_bitexact, load_golden, oracle_for


def _workload(d, nlin, nprog, seed):
    rng = np.random.default_rng(seed)
    ncol = 33   # 32 features + target: 600k records are 79 MB of columns
    rows = rng.normal(0.0, 1.0, (nlin, ncol)).astype(np.float32)
    rows[:, -1] = (rows[:, 0] * rows[:, 1] + np.sin(rows[:, 2])).astype(np.float32)
    gen = ProgramGen(d, rng, ncol)
    progs = [gen.random(int(k)) for k in rng.integers(2, 40, nprog)]
    ph, ep, sz = ProgramGen.rows(progs, d["max_size"])
    sz[3] = 0   # an empty program among them
    return rows, ph, ep, sz


@pytest.mark.gpu
@pytest.mark.parametrize("math", ["fast", "parity"])
def test_chunked_equals_unchunked(gpu_lib, math):
    import ppi_gpu
    d = load_golden("random")
    rows, ph, ep, sz = _workload(d, 600_000, 300, 7)
    ev = ppi_gpu.Evaluator(d["symtab"], d["max_size"], len(sz), "PDP", 0, d["ef"], None,
                           bool(d["reduce_max"]), bool(d["protected"]), math)
    ev.set_dataset(rows)
    block, _, chunks = ev.geometry()
    assert chunks > 1, "the dataset should be evaluated in record chunks"
    fit, best = ev.evaluate(ph, ep, sz, 0.0)   # the batch runs with alpha 0
    ev.close()
    be = ppi_gpu.BatchEvaluator(d["symtab"], d["max_size"],
                                [dict(rows=rows, n=len(sz), strategy="PDP", error_fn=d["ef"],
                                      reduce_max=bool(d["reduce_max"]),
                                      protected=bool(d["protected"]))], math)
    fit_b, best_b = be.evaluate(ph, ep, sz)
    be.close()
    assert_bitexact(fit, fit_b, "chunked vs unchunked (%s)" % math)
    assert int(best) == int(best_b[0])


@pytest.mark.gpu
def test_chunked_groups_equal_unchunked(gpu_lib):
    """More programs than one group's lane states fit in a quarter of L2: the
    items walk the groups in turn (chunk-major within each, the last group
    smaller), every program's chunks still in record order."""
    import ppi_gpu
    import torch
    d = load_golden("random")
    n = 40_000   # most of them wide-pass programs
    l2 = getattr(torch.cuda.get_device_properties(0), "L2_cache_size", 128 << 20)
    assert n > (l2 // 4) // (9 * 128 * 4), "the population should span several program groups"
    rows, ph, ep, sz = _workload(d, 600_000, n, 13)
    ev = ppi_gpu.Evaluator(d["symtab"], d["max_size"], n, "PDP", 0, d["ef"], None,
                           bool(d["reduce_max"]), bool(d["protected"]), "fast")
    ev.set_dataset(rows)
    assert ev.geometry()[2] > 1
    fit, best = ev.evaluate(ph, ep, sz, 0.0)
    ev.close()
    be = ppi_gpu.BatchEvaluator(d["symtab"], d["max_size"],
                                [dict(rows=rows, n=n, strategy="PDP", error_fn=d["ef"],
                                      reduce_max=bool(d["reduce_max"]),
                                      protected=bool(d["protected"]))], "fast")
    fit_b, best_b = be.evaluate(ph, ep, sz)
    be.close()
    assert_bitexact(fit, fit_b, "grouped chunks vs unchunked")
    assert int(best) == int(best_b[0])


@pytest.mark.gpu
def test_chunked_parity_against_oracle(gpu_lib):
    import ppi_gpu
    from oracle import pyoracle
    pyoracle.build()
    d = load_golden("random")
    rows, ph, ep, sz = _workload(d, 600_000, 24, 11)
    ev = ppi_gpu.Evaluator(d["symtab"], d["max_size"], len(sz), "PDP", 0, d["ef"], None,
                           bool(d["reduce_max"]), bool(d["protected"]), "parity")
    ev.set_dataset(rows)
    assert ev.geometry()[2] > 1
    fit, _ = ev.evaluate(ph, ep, sz, 0.0)
    ev.close()
    o = oracle_for(pyoracle, d, rows=rows)
    ref = o.evaluate(ph, ep, sz, "PDP", 1024, 0.0)
    assert_bitexact(fit, ref, "chunked vs oracle")


@pytest.mark.gpu
def test_small_dataset_is_not_chunked(gpu_lib):
    import ppi_gpu
    d = load_golden("random")
    ev = ppi_gpu.Evaluator(d["symtab"], d["max_size"], len(d["size"]), "PDP", 0, d["ef"], None,
                           bool(d["reduce_max"]), bool(d["protected"]), "fast")
    ev.set_dataset(d["rows"])
    assert ev.geometry()[2] == 1
    ev.close()
