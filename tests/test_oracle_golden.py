"""Pins the CPU oracle to the reference: every fixture was produced by the
reference's own decode, sequential interpreter and OpenCL kernels
(tests/golden/make_golden.py); the oracle must reproduce them bit for bit."""
import numpy as np
import pytest

from helpers import Tables, assert_bitexact, golden_names, load_golden, oracle_for

NAMES = golden_names()


@pytest.mark.parametrize("name", NAMES)
def test_decode_matches_reference(oracle_lib, name):
    d = load_golden(name)
    ph, ep, sz = oracle_lib.decode(Tables(d), d["genomes_bits"], d["bg"], d["bc"], -10.0, 10.0,
                                   d["max_size"])
    ref_sz = d["ref_size"].copy()
    ref_sz[ref_sz > d["max_size"]] = 0        # written past max_size: invalid here
    np.testing.assert_array_equal(sz, ref_sz)
    for i in range(len(sz)):
        if d["size"][i] > 0:
            np.testing.assert_array_equal(ph[i, :sz[i]], d["phenotype"][i, :sz[i]])
            c = (ph[i, :sz[i]] == d["t_const"]) | (ph[i, :sz[i]] == d["t_attribute"])
            assert_bitexact(ep[i, :sz[i]][c], d["ephemeral"][i, :sz[i]][c], "ephemeral %d" % i)


@pytest.mark.parametrize("name", NAMES)
def test_sequential_fitness_bitexact(oracle_lib, name):
    d = load_golden(name)
    o = oracle_for(oracle_lib, d)
    f = o.evaluate(d["phenotype"], d["ephemeral"], d["size"], "PP", 1, float(d["alpha"]))
    assert_bitexact(f, d["seq_fitness"], name)
    assert oracle_lib.best_index(f) == d["seq_best"]


@pytest.mark.parametrize("name", NAMES)
def test_predictions_bitexact(oracle_lib, name):
    d = load_golden(name)
    o = oracle_for(oracle_lib, d)
    for k, i in enumerate(d["pred_index"]):
        p = o.predict(d["phenotype"][i], d["ephemeral"][i], d["size"][i])
        assert_bitexact(p, d["seq_pred"][k], "%s program %d" % (name, i))


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("strat,lanes", [("PP", 16), ("PDP", 64), ("PDP", 7), ("DP", 32), ("DP", 5)])
def test_opencl_strategies_bitexact(oracle_lib, name, strat, lanes):
    d = load_golden(name)
    o = oracle_for(oracle_lib, d, float_math=True)
    f = o.evaluate(d["phenotype"], d["ephemeral"], d["size"], strat,
                   1 if strat == "PP" else lanes, float(d["alpha"]))
    assert_bitexact(f, d["cl_%s_%d_fitness" % (strat, lanes)], "%s %s%d" % (name, strat, lanes))


def test_best_index_ties_go_to_largest_index(oracle_lib):
    f = np.array([3, 1, 2, 1, 5, 1, 9], np.float32)
    assert oracle_lib.best_index(f) == 5


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("strat,lanes", [("PP", 16), ("PDP", 64), ("PDP", 7), ("DP", 32), ("DP", 5)])
def test_accelerator_best_index_matches_reference_kernels(oracle_lib, name, strat, lanes):
    """best_individual (work-groups of 16) + PickNBest over the alpha-free
    values (PP, PDP) or the alpha-included fitness (DP), against the index the
    reference's own kernels returned for the fixture."""
    d = load_golden(name)
    o = oracle_for(oracle_lib, d, float_math=True)
    L = 1 if strat == "PP" else lanes
    alpha = float(d["alpha"]) if strat == "DP" else 0.0
    vals = o.evaluate(d["phenotype"], d["ephemeral"], d["size"], strat, L, alpha)
    assert oracle_lib.best_index_accelerator(vals, 16) == int(d["cl_%s_%d_best" % (strat, lanes)])


def test_accelerator_best_index_tree_order(oracle_lib):
    """The strided tree keeps the left value on ties, so among equal values
    the winner is not always the smallest index: with groups of 4, values
    (5, 1, 1, 9) reduce as min(v0, v2) = v2 and min(v1, v3) = v1, then v2
    (left) beats v1.  Across groups, ties go to the last group."""
    v = np.array([5, 1, 1, 9], np.float32)
    assert oracle_lib.best_index_accelerator(v, 4) == 2
    v = np.array([2, 0, 3, 3, 0, 7, 7, 7], np.float32)
    assert oracle_lib.best_index_accelerator(v, 4) == 4
    assert oracle_lib.best_index_accelerator(v, 1) == oracle_lib.best_index(v) == 4
