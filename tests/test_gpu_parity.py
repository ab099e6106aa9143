"""GPU evaluator vs the reference (golden fixtures) and the pinned oracle.

PARITY math reproduces sequential.cc's arithmetic (double libm for the
transcendental opcodes), so its fitness and predictions must be bit-identical
to the reference for every strategy's accumulation order.  FAST math uses
CUDA's single-precision functions; its fitness is compared within a stated
relative tolerance."""
import numpy as np
import pytest

from helpers import (Tables, assert_bitexact, expected_best, golden_names, load_golden,
                     make_evaluator, oracle_for)

pytestmark = pytest.mark.gpu
NAMES = golden_names()
# Fast-math fitness tolerance (relative, finite values): CUDA's float functions
# are within 1-4 ulp of the correctly rounded result; a program's value can
# amplify that, so the sum over records is compared at 1e-4.
FAST_RTOL = 1e-4


@pytest.mark.parametrize("name", NAMES)
def test_pp_parity_equals_sequential_reference(gpu_lib, name):
    d = load_golden(name)
    ev = make_evaluator(d, "PP", 0, "parity", best_rule="sequential")
    f, best = ev.evaluate(d["phenotype"], d["ephemeral"], d["size"], float(d["alpha"]))
    assert_bitexact(f, d["seq_fitness"], name)
    assert best == d["seq_best"]


# The fixtures' cl_<strategy>_<lanes>_best are the indices the reference's own
# evaluate_* and best_individual kernels (work-groups of 16) and its host
# PickNBest returned on these programs.
CL_CASES = [("PP", 16), ("PDP", 64), ("PDP", 7), ("DP", 32), ("DP", 5)]


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("strat,lanes", CL_CASES)
def test_best_index_equals_accelerator_reference(gpu_lib, name, strat, lanes):
    d = load_golden(name)
    ev = make_evaluator(d, strat, 0 if strat == "PP" else lanes, "parity", best_group=16)
    _, best = ev.evaluate(d["phenotype"], d["ephemeral"], d["size"], float(d["alpha"]))
    assert best == int(d["cl_%s_%d_best" % (strat, lanes)]), (name, strat, lanes)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("strat,lanes", [("PDP", 64), ("PDP", 7), ("DP", 32), ("DP", 5), ("PDP", 0)])
def test_strategy_orders_bitexact(gpu_lib, oracle_lib, name, strat, lanes):
    d = load_golden(name)
    ev = make_evaluator(d, strat, lanes, "parity")
    f, best = ev.evaluate(d["phenotype"], d["ephemeral"], d["size"], float(d["alpha"]))
    L = ev.lanes
    ref = oracle_for(oracle_lib, d).evaluate(d["phenotype"], d["ephemeral"], d["size"], strat, L,
                                            float(d["alpha"]))
    assert_bitexact(f, ref, "%s %s%d" % (name, strat, lanes))
    o = oracle_for(oracle_lib, d)
    assert best == expected_best(oracle_lib, o, d["phenotype"], d["ephemeral"], d["size"], strat, L,
                                 float(d["alpha"]))


@pytest.mark.parametrize("name", NAMES)
def test_parity_predictions_equal_sequential_reference(gpu_lib, name):
    d = load_golden(name)
    ev = make_evaluator(d, "PDP", 0, "parity")
    for k, i in enumerate(d["pred_index"]):
        p = ev.predict(d["phenotype"][i], d["ephemeral"][i], d["size"][i])
        assert_bitexact(p, d["seq_pred"][k], "%s program %d" % (name, i))


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("math", ["fast", "native"])
def test_fast_math_within_tolerance(gpu_lib, oracle_lib, name, math):
    d = load_golden(name)
    ev = make_evaluator(d, "PDP", 64, math)
    f, _ = ev.evaluate(d["phenotype"], d["ephemeral"], d["size"], float(d["alpha"]))
    ref = oracle_for(oracle_lib, d).evaluate(d["phenotype"], d["ephemeral"], d["size"], "PDP", 64,
                                            float(d["alpha"]))
    fin = (ref < 1e30) & (f < 1e30)
    agree = (fin == ((ref < 1e30) & (f < 1e30))).mean()
    assert ((ref >= 1e30) == (f >= 1e30)).mean() >= (0.95 if math == "native" else 0.97)
    rel = np.abs(f[fin] - ref[fin]) / np.maximum(np.abs(ref[fin]), 1e-30)
    tol = FAST_RTOL if math == "fast" else 5e-2
    assert (rel <= tol).mean() >= (0.97 if math == "fast" else 0.85), (agree, np.sort(rel)[-5:])


@pytest.mark.parametrize("name", NAMES)
def test_device_decode_equals_reference(gpu_lib, name):
    d = load_golden(name)
    ev = make_evaluator(d, "PDP", 0, "parity")
    ev.set_grammar(Tables(d))
    ph, ep, sz = ev.decode(d["genomes_bits"], d["bg"], d["bc"], -10.0, 10.0)
    ref_sz = d["ref_size"].copy()
    ref_sz[ref_sz > d["max_size"]] = 0
    np.testing.assert_array_equal(sz, ref_sz)
    for i in range(len(sz)):
        n = sz[i]
        np.testing.assert_array_equal(ph[i, :n], d["phenotype"][i, :n])
        c = (ph[i, :n] == d["t_const"]) | (ph[i, :n] == d["t_attribute"])
        assert_bitexact(ep[i, :n][c], d["ephemeral"][i, :n][c], "ephemeral %d" % i)


@pytest.mark.parametrize("name", ["allops", "cfg2", "cfg5", "iris", "random"])
def test_device_decode_equals_oracle_on_random_genomes(gpu_lib, oracle_lib, name):
    """Fresh random genomes (several lengths, constant widths and ranges):
    the device decode against the oracle's, itself pinned to the reference's
    decode on such genomes."""
    d = load_golden(name)
    ev = make_evaluator(d, "PDP", 0, "parity", population=200)
    ev.set_grammar(Tables(d))
    rng = np.random.default_rng(78)
    for nb, bc, lo, hi in [(400, 8, -1.0, 1.0), (2000, 16, -10.0, 10.0), (6000, 24, -1e3, 5.0)]:
        genomes = rng.integers(0, 2, (200, nb), dtype=np.uint8)
        ph, ep, sz = ev.decode(genomes, d["bg"], bc, lo, hi)
        oph, oep, osz = oracle_lib.decode(Tables(d), genomes, d["bg"], bc, lo, hi, d["max_size"])
        np.testing.assert_array_equal(sz, osz)
        assert (sz > 0).sum() >= 20
        for i in np.nonzero(sz > 0)[0]:
            n = sz[i]
            np.testing.assert_array_equal(ph[i, :n], oph[i, :n])
            c = (ph[i, :n] == d["t_const"]) | (ph[i, :n] == d["t_attribute"])
            assert_bitexact(ep[i, :n][c], oep[i, :n][c], "%s genome %d" % (name, i))


@pytest.mark.parametrize("name", ["cfg2", "cfg5", "iris"])
def test_decode_evaluate_matches_separate_calls(gpu_lib, name):
    d = load_golden(name)
    ev = make_evaluator(d, "PP", 0, "parity")
    ev.set_grammar(Tables(d))
    f, best, sz = ev.decode_evaluate(d["genomes_bits"], d["bg"], d["bc"], -10.0, 10.0,
                                     float(d["alpha"]))
    keep = d["ref_size"] <= d["max_size"]
    keep[5] = False   # fixture row 5 was zeroed by hand
    assert_bitexact(f[keep], d["seq_fitness"][keep], name)
