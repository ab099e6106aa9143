"""Program shapes that exercise every path of the GPU evaluator: all register
slots, every ITE permutation, leaf folding on either side, the generic stack
interpreter (register need above 6, malformed programs), invalid attribute
indices, unknown symbols, size 0 / size > max_size, lane counts that do not
divide the records, one record, and tiny populations."""
import numpy as np
import pytest

from helpers import (ProgramGen, assert_bitexact, expected_best, load_golden, make_evaluator,
                     oracle_for)

pytestmark = pytest.mark.gpu


def _dataset(rng, nlin, nfeat, ef="abs"):
    X = rng.normal(0, 2, (nlin, nfeat)).astype(np.float32)
    y = (rng.integers(0, 3, nlin) if ef == "misclass" else rng.normal(0, 2, nlin)).astype(np.float32)
    return np.concatenate([X, y[:, None]], 1)


def _check(oracle_lib, d, rows, ph, ep, sz, strat, lanes, math="parity", alpha=1e-6):
    ev = make_evaluator(d, strat, lanes, math, population=len(sz), max_size=ph.shape[1], rows=rows)
    f, best = ev.evaluate(ph, ep, sz, alpha)
    L = ev.lanes
    assert L == (1 if strat == "PP" else lanes if lanes > 0 and strat == "DP" else
                 min(lanes, len(rows)) if lanes > 0 else
                 min(len(rows), 1024) if strat == "PDP" else min(1024, -(-len(rows) // 152)))
    o = oracle_for(oracle_lib, d, rows=rows)
    ref = o.evaluate(ph, ep, sz, strat, L, alpha)
    assert_bitexact(f, ref, "%s%d" % (strat, lanes))
    assert best == expected_best(oracle_lib, o, ph, ep, sz, strat, L, alpha)
    return f


@pytest.mark.parametrize("fixture", ["allops", "allops_prot", "allops_sqmax", "cfg5", "random"])
@pytest.mark.parametrize("strat,lanes", [("PDP", 0), ("PP", 0), ("DP", 48), ("PDP", 100)])
def test_random_trees(gpu_lib, oracle_lib, fixture, strat, lanes):
    d = load_golden(fixture)
    rng = np.random.default_rng(hash((fixture, strat, lanes)) % 2**32)
    rows = _dataset(rng, 777, d["rows"].shape[1] - 1, d["ef"])
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(0, 60, 150)]
    progs += [gen.full(k) for k in range(1, 8)]            # need 0..6: every slot
    progs += [gen.full(8)[:255]]                           # truncated: malformed, generic path
    ph, ep, sz = ProgramGen.rows(progs, 256)
    _check(oracle_lib, d, rows, ph, ep, sz, strat, lanes)


def test_register_need_above_slots_uses_generic_path(gpu_lib, oracle_lib):
    d = load_golden("allops")
    rng = np.random.default_rng(3)
    rows = _dataset(rng, 300, 3)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.full(8), gen.full(7), gen.full(6)]         # need 7 (generic), 6, 5
    ph, ep, sz = ProgramGen.rows(progs, 511)
    _check(oracle_lib, d, rows, ph, ep, sz, "PDP", 0)


def test_ite_all_permutations(gpu_lib, oracle_lib):
    d = load_golden("allops")
    rng = np.random.default_rng(4)
    rows = _dataset(rng, 500, 3)
    gen = ProgramGen(d, rng, rows.shape[1])
    ite = (gen.by_op[gen.G.OP["IF_THEN_ELSE"]][0], 0.0)
    progs = []
    for a in range(4):
        for b in range(4):
            for c in range(4):
                progs.append([ite] + gen.full(a) + gen.full(b) + gen.full(c))
    ph, ep, sz = ProgramGen.rows(progs, 64)
    _check(oracle_lib, d, rows, ph, ep, sz, "PDP", 0)


def test_malformed_invalid_and_edge_programs(gpu_lib, oracle_lib):
    d = load_golden("allops")
    rng = np.random.default_rng(5)
    rows = _dataset(rng, 130, 3)
    gen = ProgramGen(d, rng, rows.shape[1])
    G = gen.G
    attr = gen.by_op[G.OP["ATTRIBUTE"]][0]
    add = gen.by_op[G.OP["ADD"]][0]
    sin = gen.by_op[G.OP["SIN"]][0]
    progs = [
        [(add, 0.0)],                                  # binary with no operands
        [(add, 0.0), (attr, 0.0)],                     # one operand missing
        [(attr, 0.0), (attr, 1.0)],                    # two values left (forest)
        [(sin, 0.0)],                                  # unary with no operand
        [(attr, 7.0)],                                 # attribute index past ncol
        [(attr, -1.0)],                                # negative attribute index
        [(attr, float("nan"))],
        [(987654, 0.0)],                               # symbol outside the table
        [(add, 0.0), (987654, 0.0), (attr, 2.0)],
        [(attr, 3.0)],                                 # reads the target column
    ]
    ph, ep, sz = ProgramGen.rows(progs, 8)
    sz = np.concatenate([sz, [0, 9, -3]]).astype(np.int32)   # size 0, > max_size, negative
    ph = np.concatenate([ph, np.zeros((3, 8), np.int32)])
    ep = np.concatenate([ep, np.zeros((3, 8), np.float32)])
    for strat, lanes in [("PDP", 0), ("PP", 0), ("DP", 16), ("DP", 1000)]:
        _check(oracle_lib, d, rows, ph, ep, sz, strat, lanes)


@pytest.mark.parametrize("nlin", [1, 2, 31, 1023, 1024, 1025, 2049])
@pytest.mark.parametrize("strat,lanes", [("PDP", 0), ("PP", 0), ("DP", 0), ("PDP", 3)])
def test_record_counts(gpu_lib, oracle_lib, nlin, strat, lanes):
    d = load_golden("cfg2")
    rng = np.random.default_rng(nlin)
    rows = _dataset(rng, nlin, 1)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(0, 40, 37)]
    ph, ep, sz = ProgramGen.rows(progs, 128)
    _check(oracle_lib, d, rows, ph, ep, sz, strat, lanes)


def test_population_of_one_and_all_invalid(gpu_lib, oracle_lib):
    d = load_golden("cfg2")
    rng = np.random.default_rng(9)
    rows = _dataset(rng, 200, 1)
    ph = np.zeros((3, 16), np.int32)
    ep = np.zeros((3, 16), np.float32)
    sz = np.zeros(3, np.int32)
    f = _check(oracle_lib, d, rows, ph, ep, sz, "PDP", 0)
    assert (f == np.float32(3.4028235e38)).all()
    gen = ProgramGen(d, rng, rows.shape[1])
    ph, ep, sz = ProgramGen.rows([gen.random(5)], 16)
    _check(oracle_lib, d, rows, ph, ep, sz, "PP", 0)


def test_misclassification_and_reducemax_bitexact_in_fast_math(gpu_lib, oracle_lib):
    """Counts and maxima are order-independent: with the same per-record
    predictions fast math must reproduce them exactly.  Programs without
    transcendental ops have identical predictions in every math mode."""
    d = load_golden("cfg1")
    rng = np.random.default_rng(11)
    rows = d["rows"]
    gen = ProgramGen(d, rng, rows.shape[1])
    G = gen.G
    gen.un = []                                   # + - * / only
    gen.bi = [G.OP["ADD"], G.OP["SUB"], G.OP["MULT"], G.OP["DIV"]]
    progs = [gen.random(int(k)) for k in rng.integers(0, 30, 80)]
    ph, ep, sz = ProgramGen.rows(progs, 64)
    _check(oracle_lib, d, rows, ph, ep, sz, "PDP", 0, math="fast")

    dm = load_golden("cfg2max")
    rng = np.random.default_rng(12)
    gen = ProgramGen(dm, rng, dm["rows"].shape[1])
    gen.un = []
    gen.bi = [G.OP["ADD"], G.OP["SUB"], G.OP["MULT"], G.OP["DIV"]]
    progs = [gen.random(int(k)) for k in rng.integers(0, 30, 80)]
    ph, ep, sz = ProgramGen.rows(progs, 128)
    for strat in ("DP", "PDP", "PP"):
        _check(oracle_lib, dm, dm["rows"], ph, ep, sz, strat, 0, math="fast")


@pytest.mark.parametrize("fixture", ["allops", "allops_prot", "cfg2"])
@pytest.mark.parametrize("math", ["parity", "fast"])
def test_constant_subexpressions_fold_exactly(gpu_lib, oracle_lib, fixture, math):
    """Subtrees of constants are folded once per program by the translator,
    with the evaluator's own arithmetic; results must not change (PARITY is
    compared bit for bit, FAST too: folding uses the same device functions
    the per-record path would)."""
    d = load_golden(fixture)
    rng = np.random.default_rng(21)
    rows = _dataset(rng, 500, d["rows"].shape[1] - 1, d["ef"])
    gen = ProgramGen(d, rng, rows.shape[1])
    G = gen.G
    all_leaves = list(gen.leaf)
    const_leaves = [o for o in all_leaves if o in (G.OP["CONST"], G.OP["LITERAL"])]
    progs = []
    for k in range(120):
        gen.leaf = const_leaves if k % 3 else all_leaves
        sub = gen.random(int(rng.integers(1, 12)))
        gen.leaf = all_leaves
        other = gen.random(int(rng.integers(0, 8)))
        add = (gen.by_op[G.OP["ADD"]][0], 0.0)
        progs.append([add] + sub + other if k % 2 else sub)
    # zero / negative constants through DIV, LOG, SQRT (NaN, inf and protected values)
    cst = gen.by_op[G.OP["CONST"]][0]
    for opname in ("DIV", "LOG", "SQRT", "MOD", "POW"):
        if G.OP[opname] in gen.by_op:
            o = gen.by_op[G.OP[opname]][0]
            ar = G.op_arity(G.OP[opname])
            progs.append([(o, 0.0)] + [(cst, -2.5), (cst, 0.0)][:ar])
            progs.append([(o, 0.0)] + [(cst, 0.0), (cst, -0.0)][:ar])
    # malformed program holding a foldable subtree: goes to the generic path unfolded
    progs.append([(gen.by_op[G.OP["ADD"]][0], 0.0), (gen.by_op[G.OP["MULT"]][0], 0.0), (cst, 2.0), (cst, 3.0)][:3])
    ph, ep, sz = ProgramGen.rows(progs, 64)
    for strat in ("PDP", "PP"):
        _check(oracle_lib, d, rows, ph, ep, sz, strat, 0, math="parity")
    if math == "fast":
        # fast math against itself with folding effectively off (every constant
        # moved into a record column would change nothing; compare to parity
        # only where no transcendental is involved is done elsewhere)
        ev = make_evaluator(d, "PDP", 0, "fast", population=len(sz), max_size=64, rows=rows)
        f1, _ = ev.evaluate(ph, ep, sz, 1e-6)
        f2, _ = ev.evaluate(ph, ep, sz, 1e-6)
        assert np.array_equal(f1.view(np.int32), f2.view(np.int32))


def _sum_of_columns(gen, cols):
    """Left-deep sum of the given attribute columns (register need 0)."""
    G = gen.G
    add = gen.by_op[G.OP["ADD"]][0]
    attr = gen.by_op[G.OP["ATTRIBUTE"]][0]
    return [(add, 0.0)] * (len(cols) - 1) + [(attr, float(c)) for c in cols]


@pytest.mark.parametrize("strat,lanes", [("PDP", 0), ("PP", 0), ("DP", 64), ("DP", 7), ("DP", 5),
                                         ("DP", 6), ("DP", 301), ("PDP", 100)])
def test_wide_dataset_staged_and_direct_columns(gpu_lib, oracle_lib, strat, lanes):
    """A 90-column dataset: programs reading a few columns stage them all in
    the tile; programs reading 12-85 distinct columns stage the most-read
    ones and read the rest directly from global memory (whole 16-byte quads
    where every tile starts on a multiple of 4 records: DP tiles hold a
    whole-quad number of groups, 48 groups of 5 lanes or 42 of 6 in a tile
    of 256 slots; DP over 301 lanes steps by 301 records, so its reads take
    the ragged, scalar path).  Two evaluations in a row must both match the
    oracle bit for bit."""
    d = load_golden("allops")
    rng = np.random.default_rng(77 + lanes)
    rows = _dataset(rng, 3000, 90)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(0, 40, 60)]
    for k in (1, 5, 12, 20, 30, 40, 55, 70, 85):
        progs.append(_sum_of_columns(gen, rng.permutation(90)[:k]))
        progs.append([gen.op_tok(1)] + _sum_of_columns(gen, rng.integers(0, 90, k)))   # repeats
    rng.shuffle(progs)
    ph, ep, sz = ProgramGen.rows(progs, 200)
    # a population capacity far above one wave keeps the main tile at its
    # occupancy-driven size (a population that fits one wave gets every row it
    # can use), so the wide programs take the direct-read path
    ev = make_evaluator(d, strat, lanes, "parity", population=20000, max_size=200, rows=rows)
    o = oracle_for(oracle_lib, d, rows=rows)
    ref = o.evaluate(ph, ep, sz, strat, ev.lanes, 1e-6)
    want = expected_best(oracle_lib, o, ph, ep, sz, strat, ev.lanes, 1e-6, population=20000)
    for rep in range(2):
        f, best = ev.evaluate(ph, ep, sz, 1e-6)
        assert_bitexact(f, ref, "%s%d rep %d" % (strat, lanes, rep))
        assert best == want
    pred = ev.predict(ph[-1], ep[-1], int(sz[-1]))
    assert_bitexact(pred, oracle_for(oracle_lib, d, rows=rows).predict(ph[-1], ep[-1], int(sz[-1])),
                    "predict")


def test_large_population_thread_per_program_translator(gpu_lib, oracle_lib):
    """12,000 programs: more than one wave of warps (64 x SMs on a GB300), so
    the translator runs a thread per program with its scratch in global
    memory (smaller populations get a warp per program); bit-exact against
    the oracle, every opcode."""
    d = load_golden("allops")
    rng = np.random.default_rng(31)
    rows = _dataset(rng, 200, d["rows"].shape[1] - 1)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(0, 25, 12000)]
    ph, ep, sz = ProgramGen.rows(progs, 64)
    _check(oracle_lib, d, rows, ph, ep, sz, "PDP", 0)


def test_population_in_one_wave_runs_without_wide_pass(gpu_lib, oracle_lib):
    """A population resident in one wave gets the main tile with every row its
    programs can need (here all 4 columns, the target and the slots): the
    evaluation is the translator and one evaluator launch, bit-exact."""
    d = load_golden("allops")
    rng = np.random.default_rng(32)
    rows = _dataset(rng, 500, d["rows"].shape[1] - 1)
    gen = ProgramGen(d, rng, rows.shape[1])
    progs = [gen.random(int(k)) for k in rng.integers(0, 40, 300)]
    ph, ep, sz = ProgramGen.rows(progs, 64)
    ev = make_evaluator(d, "PDP", 0, "parity", population=len(sz), max_size=64, rows=rows)
    f, _ = ev.evaluate(ph, ep, sz, 1e-6)
    assert ev.last_launch_count() == 2
    assert_bitexact(f, oracle_for(oracle_lib, d, rows=rows).evaluate(ph, ep, sz, "PDP", ev.lanes, 1e-6),
                    "one wave")
