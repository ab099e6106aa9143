"""The oracle against the reference's own OpenCL kernels at lane counts the
fixtures do not hold (CPU; skipped where the reference was not compiled
into oracle/_ref).  The fixtures pin PP 16, PDP 64 / 7 and DP 32 / 5; the
evaluator also runs DP over group sizes that are not multiples of 4 (tiles
rounded to whole quads, or ragged when one group fills a tile) and PDP
over any lane count, and its GPU tests compare with the oracle there.
Here the oracle meets the reference's accelerator.cl (compiled as C++ by
oracle/build_ref.py) on the fixtures' programs and datasets at those lane
counts: fitness bit for bit, and the index best_individual + PickNBest
return (work-groups of 16 programs)."""
import pytest

from helpers import assert_bitexact, expected_best, load_golden, oracle_for

DP_LANES = [1, 3, 6, 7, 33, 101]   # 101: one group fills a 256-slot tile, raggedly
PDP_LANES = [3, 100]
# abs over 50 columns; every opcode with squared error and REDUCEMAX; COST
FIXTURES = ["random", "allops_sqmax", "cfg5"]


def _ref(name):
    from oracle import pyoracle
    man = pyoracle.ref_manifest()
    if name not in man:
        pytest.skip("the reference is not compiled into oracle/_ref here")
    return pyoracle.RefBuild(name)


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_equals_reference_kernels(oracle_lib, name):
    from oracle import pyoracle
    d = load_golden(name)
    ref = _ref(name)
    ph, ep, sz = d["phenotype"], d["ephemeral"], d["size"]
    alpha = float(d["alpha"])
    # the shimmed OpenCL kernels call the float math functions (the
    # sequential interpreter the double ones): the oracle's float-math mode.
    # Their work-groups run each work-item as a thread, so the lane counts
    # are kept few and small.
    o = oracle_for(pyoracle, d, float_math=True)
    nlin = d["rows"].shape[0]
    cases = [("DP", L) for L in DP_LANES] + [("PDP", L) for L in PDP_LANES]
    for strategy, lanes in [(s_, L) for s_, L in cases if L <= nlin]:
        want, want_best = ref.cl_evaluate(strategy, d["rows"], ph, ep, sz, lanes, 16, alpha=alpha)
        got = o.evaluate(ph, ep, sz, strategy, lanes, alpha)
        assert_bitexact(got, want, "%s %s %d" % (name, strategy, lanes))
        assert expected_best(oracle_lib, o, ph, ep, sz, strategy, lanes, alpha, group=16) == want_best, \
            "%s %s %d best index" % (name, strategy, lanes)
