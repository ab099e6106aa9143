"""The synthetic workloads the benchmark and the GPU tests run on (CPU): every
generated program is a well-formed prefix tree of the requested length, and the
uneven batch and the adjoint configuration have the shapes they promise."""
import numpy as np

from ppi_gpu import grammar as G
from ppi_gpu import workloads as W


def _well_formed(ops):
    """Right-to-left stack discipline of a prefix program: never short of
    operands, one value left."""
    depth = 0
    for op in reversed(ops):
        ar = G.op_arity(op)
        if depth < ar:
            return False
        depth = depth - ar + 1
    return depth == 1


def _ops(g, ph_row, n):
    s, o, _ = g.symbol_table_arrays()
    lut = dict(zip(s.tolist(), o.tolist()))
    return [lut[int(t)] for t in ph_row[:n]]


def test_random_programs_are_valid_trees_of_the_requested_length():
    g, _, _, _, _ = W.adjoint(nlin=10, population=1)
    rng = np.random.default_rng(5)
    lengths = rng.integers(1, 120, 400)
    ph, ep = W.random_programs(rng, lengths, 6, g, p_unary=0.3, lo=-1.5, hi=2.5)
    attr, const = g.symbols["T_ATTRIBUTE"], g.symbols["T_CONST"]
    for i, n in enumerate(lengths):
        assert _well_formed(_ops(g, ph[i], n)), i
        assert np.all(ph[i, n:] == 0)
        cols = ep[i, :n][ph[i, :n] == attr]
        assert np.all((cols >= 0) & (cols < 6) & (cols == np.floor(cols)))
        consts = ep[i, :n][ph[i, :n] == const]
        assert np.all((consts >= -1.5) & (consts <= 2.5))


def test_uneven_batch_shapes():
    g, pops = W.uneven_batch(seed=4, n_pops=8, pop_range=(20, 300), rec_range=(50, 5000),
                             feat_range=(2, 9), mean_len=12, len_range=(4, 64), max_size=64)
    assert len(pops) == 8
    for p in pops:
        nlin, ncol = p["rows"].shape
        assert 20 <= p["n"] <= 300 and 50 <= nlin <= 5000 and 3 <= ncol <= 10
        assert p["phenotype"].shape == (p["n"], 64) and p["size"].shape == (p["n"],)
        assert np.all((p["size"] >= 4) & (p["size"] <= 64))
        for i in range(0, p["n"], 7):
            assert _well_formed(_ops(g, p["phenotype"][i], int(p["size"][i])))


def test_adjoint_programs_have_one_to_eight_constants():
    g, rows, ph, ep, sz = W.adjoint(nlin=200, population=300)
    const = g.symbols["T_CONST"]
    assert rows.shape == (200, 9)
    for i in range(len(sz)):
        k = int((ph[i, :sz[i]] == const).sum())
        assert 1 <= k <= 8
        assert _well_formed(_ops(g, ph[i], int(sz[i])))
