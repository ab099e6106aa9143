"""Parity at the benchmark configurations' own scale, and the fast-math
error budget.

The fixtures hold 96 programs over at most 301 records; here the GPU meets the
oracle on the shapes the benchmark runs: the polynomial workload at 100k
records (PDP over 1024 lanes, sum and REDUCEMAX), a 200k-record x 32-feature
slice of the streaming workload (COST, DP and PDP), the iris-shaped
population, and an uneven batch whose datasets reach a million records.  In
parity math every fitness is bit-identical to the oracle (the same strategy's
accumulation order) and every best index is the one acc_interpret returns.

Fast math (CUDA's single-precision functions, the benchmarked mode) is held
per opcode to 2 ulp of the correctly rounded result on the arithmetic
grammars' functions, and its fitness to a stated relative bound of the
oracle; both are also compared with an FP64 re-evaluation."""
import numpy as np
import pytest

from helpers import assert_bitexact, expected_best

pytestmark = pytest.mark.gpu


def _decode(wl):
    from oracle import pyoracle
    return pyoracle.decode(wl.grammar, wl.genomes, wl.bits_per_gene, wl.bits_per_constant, wl.lo,
                           wl.hi, wl.max_size)


def _evaluator(wl, strategy, lanes, math, n, reduce_max=None):
    import ppi_gpu
    ev = ppi_gpu.Evaluator(wl.grammar.symbol_table_arrays(), wl.max_size, n, strategy, lanes,
                           wl.error_fn, wl.cost, wl.reduce_max if reduce_max is None else reduce_max,
                           wl.protected, math)
    ev.set_dataset(wl.rows)
    return ev


def _oracle(wl, float_math=False):
    from oracle import pyoracle
    return pyoracle.Oracle(wl.rows, wl.grammar.symbol_table_arrays(), wl.error_fn, wl.cost,
                           wl.reduce_max, wl.protected, float_math)


def _parity_case(oracle_lib, wl, strategy, lanes, n):
    ph, ep, sz = _decode(wl)
    ph, ep, sz = ph[:n], ep[:n], sz[:n]
    ev = _evaluator(wl, strategy, lanes, "parity", n)
    f, best = ev.evaluate(ph, ep, sz, 1e-6)
    o = _oracle(wl)
    ref = o.evaluate(ph, ep, sz, strategy, ev.lanes, 1e-6)
    assert_bitexact(f, ref, "%s %s%d" % (wl.name, strategy, lanes))
    assert best == expected_best(oracle_lib, o, ph, ep, sz, strategy, ev.lanes, 1e-6)
    assert (f < 1e30).sum() >= n // 4   # most programs are valid and finite
    lanes = ev.lanes
    ev.close()
    return lanes


@pytest.mark.parametrize("reduce_max", [False, True])
def test_polynomial_100k_pdp_1024_lanes_bitexact(gpu_lib, oracle_lib, reduce_max):
    from ppi_gpu import workloads
    wl = workloads.polynomial(seed=1234, nlin=100_000, population=200, reduce_max=reduce_max)
    assert _parity_case(oracle_lib, wl, "PDP", 0, 200) == 1024


@pytest.mark.parametrize("strategy,lanes", [("PDP", 0), ("DP", 0), ("DP", 40)])
def test_streaming_200k_x32_cost_bitexact(gpu_lib, oracle_lib, strategy, lanes):
    from ppi_gpu import workloads
    wl = workloads.streaming(seed=7, nlin=200_000, population=120)
    _parity_case(oracle_lib, wl, strategy, lanes, 120)


def test_iris_population_pp_bitexact(gpu_lib, oracle_lib):
    from ppi_gpu import workloads
    wl = workloads.iris_shaped(seed=99, population=1000)
    _parity_case(oracle_lib, wl, "PP", 0, 1000)


def test_uneven_batch_up_to_a_million_records_bitexact(gpu_lib, oracle_lib):
    """Eight populations of the uneven-batch generator with their full record
    counts (up to 1M) and a few dozen programs each, in one batched launch."""
    import ppi_gpu
    from oracle import pyoracle
    from ppi_gpu import workloads
    g, pops = workloads.uneven_batch(seed=12, n_pops=8, pop_range=(16, 48),
                                     rec_range=(20_000, 1_000_000))
    assert max(p["rows"].shape[0] for p in pops) > 800_000
    sym = g.symbol_table_arrays()
    ph = np.concatenate([p["phenotype"] for p in pops])
    ep = np.concatenate([p["ephemeral"] for p in pops])
    sz = np.concatenate([p["size"] for p in pops])
    be = ppi_gpu.BatchEvaluator(sym, ph.shape[1], pops, "parity")
    fit, best = be.evaluate(ph, ep, sz, ppi_gpu.BATCH_GRAPH)
    begin = 0
    for k, p in enumerate(pops):
        sl = slice(begin, begin + p["n"])
        o = pyoracle.Oracle(p["rows"], sym, "abs", None, False, True, False)
        lanes = min(p["rows"].shape[0], 1024)
        ref = o.evaluate(p["phenotype"], p["ephemeral"], p["size"], "PDP", lanes, 0.0)
        assert_bitexact(fit[sl], ref, "population %d (%d records)" % (k, p["rows"].shape[0]))
        assert best[k] == expected_best(oracle_lib, o, p["phenotype"], p["ephemeral"], p["size"],
                                        "PDP", lanes, 0.0)
        begin += p["n"]
    be.close()


# ---- fast math -------------------------------------------------------------

def _ulp_distance(a, b):
    """Units in the last place between float32 arrays (same-sign ordering;
    equal infinities and NaN pairs count 0)."""
    ai = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    bi = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7FFFFFFF), ai)
    bi = np.where(bi < 0, -(bi & 0x7FFFFFFF), bi)
    d = np.abs(ai - bi)
    d[np.isnan(a) & np.isnan(b)] = 0
    return d


# Inputs per opcode family: a wide range and the function's own domain.
def _inputs(rng, op, n):
    wide = np.concatenate([rng.uniform(-20, 20, n // 2), rng.uniform(-1e4, 1e4, n // 4),
                           rng.normal(0, 1, n - n // 2 - n // 4)])
    if op in ("LOG", "LOG2", "LOG10", "SQRT"):
        return np.abs(wide) + rng.uniform(0, 2, n)
    if op in ("EXP", "EXP2", "EXP10", "LOGISTIC", "GAUSS"):
        return rng.uniform(-30, 30, n)
    return wide


# 2 ulp for the functions of the arithmetic grammars (the benchmarked ones);
# the others at the bound measured here, each a single CUDA routine except
# the compound GAMMA (sinh, pow and two square roots).
ULP_BOUND = {"SIN": 2, "COS": 2, "EXP": 2, "LOG": 2, "SQRT": 0, "ABS": 0, "NEG": 0, "POW2": 0,
             "EXP2": 2, "EXP10": 2, "LOG2": 2, "LOG10": 2, "TAN": 4, "LOGISTIC": 4, "GAUSS": 2,
             "GAMMA": 64, "ADD": 0, "SUB": 0, "MULT": 0, "DIV": 0, "POW": 8, "MOD": 0, "MEAN": 0}


@pytest.mark.parametrize("op", sorted(ULP_BOUND))
def test_fast_math_prediction_ulp_per_opcode(gpu_lib, op):
    """One-opcode programs over 4096 random records: FAST predictions against
    the oracle's sequential.cc arithmetic (double libm rounded to float, the
    correctly rounded value but for rare double roundings)."""
    import ppi_gpu
    from oracle import pyoracle
    from ppi_gpu import grammar as G
    rng = np.random.default_rng(abs(hash(op)) % 2**32)
    n = 4096
    x0 = _inputs(rng, op, n).astype(np.float32)
    x1 = (np.abs(_inputs(rng, op, n)) + 0.25 if op in ("POW", "MOD", "DIV") else
          _inputs(rng, op, n)).astype(np.float32)
    if op == "POW":
        x0 = np.abs(x0) + 0.5
        x1 = rng.uniform(-4, 4, n).astype(np.float32)
    rows = np.stack([x0, x1, np.zeros(n, np.float32)], 1)
    # symbol table: attributes, and the op under test
    sv = np.array([10000, 10001], np.int32)
    so = np.array([G.OP["ATTRIBUTE"], G.OP[op]], np.int32)
    sl = np.zeros(2, np.float32)
    arity = G.op_arity(G.OP[op])
    ph = np.zeros((1, 4), np.int32)
    ep = np.zeros((1, 4), np.float32)
    toks = [10001] + [10000] * arity
    ph[0, :len(toks)] = toks
    ep[0, 1:1 + arity] = np.arange(arity)
    for prot in (False, True):
        ev = ppi_gpu.Evaluator((sv, so, sl), 4, 1, "PDP", 0, "abs", None, False, prot, "fast")
        ev.set_dataset(rows)
        got = ev.predict(ph[0], ep[0], len(toks))
        ev.close()
        o = pyoracle.Oracle(rows, (sv, so, sl), "abs", None, False, prot, False)
        ref = o.predict(ph[0], ep[0], len(toks))
        both_finite = np.isfinite(ref) & np.isfinite(got)
        same_class = (np.isnan(ref) == np.isnan(got)) & (np.isinf(ref) == np.isinf(got))
        assert same_class.mean() >= 0.999, (op, prot)
        d = _ulp_distance(got[both_finite], ref[both_finite])
        assert d.max() <= ULP_BOUND[op], (op, prot, int(d.max()), x0[both_finite][d.argmax()])


def test_fast_math_fitness_at_polynomial_scale(gpu_lib, oracle_lib):
    """FAST fitness of 300 decoded polynomial programs over 100k records
    against the oracle (sequential arithmetic, same PDP order) and FP64.
    Measured on a GB300: sentinels agree; the median program within 1e-6
    relative; 96.9% within 1e-5; the largest difference 1.5e-2.  The
    per-record predictions differ by a few ulp (the per-opcode test above);
    a program whose value is a large quantity nearly cancelled, or a steep
    function of one, turns those ulp into a larger relative change of its
    error, so the 1e-5 bound holds for most programs, not all, and the test
    states the measured shares."""
    from ppi_gpu import workloads
    wl = workloads.polynomial(seed=1234, nlin=100_000, population=300)
    ph, ep, sz = _decode(wl)
    ev = _evaluator(wl, "PDP", 0, "fast", len(sz))
    f, _ = ev.evaluate(ph, ep, sz, 0.0)
    o = _oracle(wl)
    ref = o.evaluate(ph, ep, sz, "PDP", ev.lanes, 0.0)
    f64 = o.evaluate64(ph, ep, sz)
    fin = (ref < 1e30) & (f < 1e30)
    assert ((ref >= 1e30) == (f >= 1e30)).mean() >= 0.99
    rel = np.abs(f[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1e-30)
    assert np.median(rel) <= 1e-6
    assert (rel <= 1e-5).mean() >= 0.95, np.sort(rel)[-5:]
    assert (rel <= 1e-3).mean() >= 0.98 and rel.max() <= 5e-2, np.sort(rel)[-5:]
    ok = fin & np.isfinite(f64)
    rel64 = np.abs(f[ok] - f64[ok]) / np.maximum(np.abs(f64[ok]), 1e-30)
    assert np.median(rel64) <= 1e-5
    ev.close()
