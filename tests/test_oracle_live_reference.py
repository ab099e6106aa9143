"""The oracle against the reference's own OpenCL kernels at lane counts the
fixtures do not hold (CPU; skipped where the reference was not compiled
into oracle/_ref).  The fixtures pin PP 16, PDP 64 / 7 and DP 32 / 5; the
evaluator also runs DP over group sizes that are not multiples of 4 (tiles
rounded to whole quads, or ragged when one group fills a tile) and PDP
over any lane count, and its GPU tests compare with the oracle there.
Here the oracle meets the reference's accelerator.cl (compiled as C++ by
oracle/build_ref.py) on the fixtures' programs and datasets at those lane
counts: fitness bit for bit, and the index best_individual + PickNBest
return (work-groups of 16 programs).

The fixtures also hold 96 decoded programs each; random programs from the
tests' generator (every opcode of the grammar, nesting up to 60 operators,
within max_size) add the reference's sequential interpreter (fitness, best
index, predictions) and its OpenCL kernels at the fixtures' own lane
counts.  And genome decode on fresh random genomes of several lengths,
bits per gene and constant ranges."""
import numpy as np
import pytest

from helpers import ProgramGen, Tables, assert_bitexact, expected_best, load_golden, oracle_for

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


def _random_programs(d, n, seed):
    rng = np.random.default_rng(seed)
    gen = ProgramGen(d, rng, d["rows"].shape[1])
    progs = []
    while len(progs) < n:
        p = gen.random(int(rng.integers(0, 60)))
        if len(p) <= d["max_size"]:   # whole programs: the reference reads no missing operand
            progs.append(p)
    return ProgramGen.rows(progs, d["max_size"])


@pytest.mark.parametrize("name", ["allops", "allops_prot", "allops_sqmax", "cfg5", "random"])
def test_oracle_equals_reference_on_random_programs(oracle_lib, name):
    from oracle import pyoracle
    d = load_golden(name)
    ref = _ref(name)
    ph, ep, sz = _random_programs(d, 300, 2026)
    alpha = float(d["alpha"])
    # the sequential interpreter (double libm): the oracle's default arithmetic
    want, want_best = ref.seq_evaluate(d["rows"], ph, ep, sz, alpha=alpha)
    o = oracle_for(pyoracle, d)
    got = o.evaluate(ph, ep, sz, "PP", 1, alpha)
    assert_bitexact(got, want, "%s sequential" % name)
    assert oracle_lib.best_index(got) == want_best
    for i in range(0, len(sz), 50):
        p_, _ = ref.seq_evaluate(d["rows"], ph[i:i + 1], ep[i:i + 1], sz[i:i + 1], prediction=True)
        assert_bitexact(o.predict(ph[i], ep[i], sz[i]), p_, "%s prediction %d" % (name, i))
    # the OpenCL kernels (float math functions) at the fixtures' lane counts
    of = oracle_for(pyoracle, d, float_math=True)
    for strategy, lanes in [("PP", 16), ("PDP", 7), ("DP", 5)]:
        want, want_best = ref.cl_evaluate(strategy, d["rows"], ph, ep, sz, lanes, 16, alpha=alpha)
        assert_bitexact(of.evaluate(ph, ep, sz, strategy, lanes, alpha), want,
                        "%s %s %d" % (name, strategy, lanes))
        assert expected_best(oracle_lib, of, ph, ep, sz, strategy, lanes, alpha, group=16) == want_best


@pytest.mark.parametrize("name", ["allops", "cfg2", "cfg5", "iris", "random"])
def test_oracle_decode_equals_reference_on_random_genomes(oracle_lib, name):
    d = load_golden(name)
    ref = _ref(name)
    rng = np.random.default_rng(77)
    ms = d["max_size"]
    for nb, bg, bc, lo, hi in [(400, d["bg"], 8, -1.0, 1.0), (2000, d["bg"], 16, -10.0, 10.0),
                               (6000, d["bg"], 24, -1e3, 5.0)]:
        genomes = rng.integers(0, 2, (200, nb), dtype=np.uint8)
        rph, rep, rsz, _ = ref.decode(genomes, bg, bc, lo, hi, ms)
        ph, ep, sz = oracle_lib.decode(Tables(d), genomes, bg, bc, lo, hi, ms)
        want = rsz.copy()
        want[want > ms] = 0   # the reference wrote past max_size: invalid here
        np.testing.assert_array_equal(sz, want)
        assert (sz > 0).sum() >= 50, "most genomes should decode to programs"
        for i in np.nonzero(sz > 0)[0]:
            np.testing.assert_array_equal(ph[i, :sz[i]], rph[i, :sz[i]])
            c = (ph[i, :sz[i]] == d["t_const"]) | (ph[i, :sz[i]] == d["t_attribute"])
            assert_bitexact(ep[i, :sz[i]][c], rep[i, :sz[i]][c], "%s genome %d" % (name, i))
