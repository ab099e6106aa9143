"""The oracle's FP64 re-evaluation (ppio_evaluate64), the yardstick the float
evaluators' error is stated against: it agrees exactly with the FP64 adjoint's
fitness (a separate double-precision walk over the same programs), and the
reference's float results stay close to it wherever both are finite."""
import numpy as np
import pytest

from helpers import golden_names, load_golden, oracle_for

NAMES = golden_names()


@pytest.mark.parametrize("name", NAMES)
def test_fp64_fitness_equals_adjoint_fp64_fitness(oracle_lib, name):
    d = load_golden(name)
    if d["ef"] not in ("abs", "squared") or d["reduce_max"]:
        pytest.skip("the FP64 adjoint covers the absolute and squared sums only")
    o = oracle_for(oracle_lib, d)
    f64 = o.evaluate64(d["phenotype"], d["ephemeral"], d["size"])
    a64, _ = o.adjoint64(d["phenotype"], d["ephemeral"].astype(np.float64), d["size"])
    both = np.isfinite(f64) & np.isfinite(a64)
    np.testing.assert_array_equal(f64[both], a64[both])
    # every non-finite FP64 fitness is a size-0/non-finite program for the adjoint too
    assert (np.isinf(f64) == (np.isinf(a64) | np.isnan(a64)))[d["size"] > 0].mean() > 0.9


@pytest.mark.parametrize("name", NAMES)
def test_reference_float_fitness_near_fp64(oracle_lib, name):
    """The reference's sequential float fitness against FP64: the median
    program within 1e-6 relative (float rounding), every program within 5e-2
    (amplified cases: near-cancelling predictions, classes flipped by a
    rounding)."""
    d = load_golden(name)
    o = oracle_for(oracle_lib, d)
    f32 = d["seq_fitness"].astype(np.float64) - float(d["alpha"]) * d["size"]
    f64 = o.evaluate64(d["phenotype"], d["ephemeral"], d["size"])
    ok = (d["seq_fitness"] < 1e30) & np.isfinite(f64)
    rel = np.abs(f32[ok] - f64[ok]) / np.maximum(np.abs(f64[ok]), 1e-30)
    assert np.median(rel) <= 1e-6
    assert rel.max() <= 5e-2


def test_fp64_misclass_and_max_reduction(oracle_lib):
    """Hand-checkable: a one-token program x0 against labels, as a
    misclassification count and as REDUCEMAX of the absolute error."""
    from oracle import pyoracle
    rows = np.array([[1, 1], [2, 3], [3, 3], [4, 0]], np.float32)
    sym = (np.array([10000], np.int32), np.array([1], np.int32), np.array([0], np.float32))
    ph = np.array([[10000]], np.int32)
    ep = np.array([[0.0]], np.float32)
    sz = np.array([1], np.int32)
    mis = pyoracle.Oracle(rows, sym, "misclass").evaluate64(ph, ep, sz)
    assert mis[0] == 2 / 4
    mx = pyoracle.Oracle(rows, sym, "abs", reduce_max=True).evaluate64(ph, ep, sz)
    assert mx[0] == 4 * 4 / 4      # max |x - y| = 4, times nlin, over nlin
