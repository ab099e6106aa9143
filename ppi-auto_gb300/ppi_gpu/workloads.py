"""Seeded synthetic workloads shaped like the benchmark configurations.

No public dataset is involved: each workload draws its records and genomes
from a fixed seed with the shapes and value distributions of the named
configuration.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

from . import grammar as G

GRAMMARS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "grammars")


@dataclasses.dataclass
class Workload:
    name: str
    rows: np.ndarray          # nlin x ncol float32, target last
    grammar: G.Grammar
    genomes: np.ndarray       # pop x nb uint8 (0/1)
    bits_per_gene: int
    bits_per_constant: int
    lo: float
    hi: float
    max_size: int
    error_fn: str
    protected: bool
    reduce_max: bool
    strategy: str
    cost: np.ndarray | None = None

    @property
    def nlin(self):
        return self.rows.shape[0]

    @property
    def population(self):
        return self.genomes.shape[0]

    def describe(self):
        return {"workload": self.name, "records": int(self.nlin),
                "features": int(self.rows.shape[1] - 1), "population": int(self.population),
                "max_size": int(self.max_size), "strategy": self.strategy,
                "error_fn": self.error_fn, "reduce_max": bool(self.reduce_max),
                "protected": bool(self.protected)}


def _grammar_setup(path, nb, mps):
    g = G.load(path)
    bg = G.effective_bits_per_gene(g, 8)
    return g, bg, G.max_phenotype_size(g, nb, bg, mps)


def polynomial(seed=1234, nlin=100_000, population=30_000, reduce_max=False, nb=2000):
    """Polynomial regression, PDP: x0 ~ U[-5, 5], y = degree-4 polynomial with
    N(0, 1) coefficients + N(0, 0.01) noise; programs <= 128 opcodes from the
    arithmetic grammar plus ^2; EF fabs((X)-(Y)), protected functions."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-5.0, 5.0, nlin)
    coef = rng.normal(0.0, 1.0, 5)
    y = sum(coef[k] * x ** k for k in range(5)) + rng.normal(0.0, 0.01, nlin)
    rows = np.stack([x, y], 1).astype(np.float32)
    g, bg, mps = _grammar_setup(os.path.join(GRAMMARS, "config2_poly.bnf"), nb, 128)
    genomes = rng.integers(0, 2, (population, nb), dtype=np.uint8)
    return Workload("polynomial-%dk-pop%d%s" % (nlin // 1000, population,
                                                "-reducemax" if reduce_max else ""),
                    rows, g, genomes, bg, 16, -10.0, 10.0, mps, "abs", True, reduce_max, "PDP")


def iris_shaped(seed=99, population=1000, nb=2000):
    """Iris-shaped classification, PP: 150 records x 4 features uniform in
    [4,8], [2,4.5], [1,7], [0.1,2.5], labels {0,1,2}; programs <= 64 opcodes;
    EF ((X)!=(Y)), sum."""
    rng = np.random.default_rng(seed)
    lo = np.array([4, 2, 1, 0.1])
    hi = np.array([8, 4.5, 7, 2.5])
    X = lo + (hi - lo) * rng.random((150, 4))
    y = rng.integers(0, 3, 150)
    rows = np.concatenate([X, y[:, None]], 1).astype(np.float32)
    g, bg, mps = _grammar_setup(os.path.join(GRAMMARS, "config1_iris.bnf"), nb, 64)
    genomes = rng.integers(0, 2, (population, nb), dtype=np.uint8)
    return Workload("iris-150-pop%d" % population, rows, g, genomes, bg, 16, -10.0, 10.0, mps,
                    "misclass", True, False, "PP")


def cost_matrix8(seed=5):
    """Seeded 8x8 cost matrix: 0 diagonal, off-diagonal uniform [0.5, 2]."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.5, 2.0, (8, 8)).astype(np.float32)
    np.fill_diagonal(c, 0.0)
    return c


def streaming(seed=7, nlin=4_000_000, population=30_000, nb=4000, native=False):
    """Large streaming classification: nlin x 32 features N(0,1) with 5% drawn
    from N(0,100); 8 classes = argmax of 8 random projections; programs <= 256
    opcodes; EF COST[(int)X][(int)Y] (guarded) with an 8x8 cost matrix."""
    rng = np.random.default_rng(seed)
    X = rng.normal(0.0, 1.0, (nlin, 32)).astype(np.float32)
    out = rng.random((nlin, 32)) < 0.05
    X[out] = rng.normal(0.0, 100.0, int(out.sum())).astype(np.float32)
    W = rng.normal(0.0, 1.0, (32, 8)).astype(np.float32)
    y = np.argmax(X @ W, 1).astype(np.float32)
    rows = np.concatenate([X, y[:, None]], 1)
    g, bg, mps = _grammar_setup(os.path.join(GRAMMARS, "config5_stream.bnf"), nb, 256)
    genomes = rng.integers(0, 2, (population, nb), dtype=np.uint8)
    return Workload("stream-%dk-x32-pop%d" % (nlin // 1000, population), rows, g, genomes, bg, 16,
                    -10.0, 10.0, mps, "cost", True, False, "PDP", cost=cost_matrix8())


BUILDERS = {"polynomial": polynomial, "iris": iris_shaped, "stream": streaming}


def random_programs(rng, lengths, ncol, grammar, p_unary=0.2, lo=-10.0, hi=10.0):
    """Random valid prefix programs of the given lengths over the arithmetic
    grammar's symbols (+ - * / and its unary ops; leaves: attributes and
    constants).  Each program is a random sequence of node arities with one
    more leaf than binary nodes, rotated to its unique valid start (the cycle
    lemma), so every length gives a well-formed tree.  Returns
    (phenotype, ephemeral) rows of max(lengths) entries."""
    S = grammar.symbols
    binary = [S[k] for k in ("T_ADD", "T_SUB", "T_MULT", "T_DIV") if k in S]
    unary = [S[k] for k in ("T_SIN", "T_COS", "T_EXP", "T_LOG", "T_SQRT", "T_POW2") if k in S]
    attr, const = S["T_ATTRIBUTE"], S["T_CONST"]
    n = len(lengths)
    width = int(max(lengths))
    ph = np.zeros((n, width), np.int32)
    ep = np.zeros((n, width), np.float32)
    for k in np.unique(lengths):
        idx = np.flatnonzero(lengths == k)
        m = len(idx)
        # node counts: u unary, b binary, b + 1 leaves, 2b + 1 + u = k
        u = np.minimum(rng.binomial(k, p_unary, m), (k - 1))
        odd = (k - 1 - u) % 2                # k - 1 - u must be even
        u = np.where(u - odd >= 0, u - odd, u + odd)
        b = (k - 1 - u) // 2
        pos = np.arange(k)[None, :]
        arity = np.where(pos < b[:, None], 2, np.where(pos < (b + u)[:, None], 1, 0))
        arity = np.take_along_axis(arity, np.argsort(rng.random((m, k)), 1), 1)
        # Read right to left, a prefix program is valid when every running
        # sum of (1 - arity) is >= 1.  In the reversed sequence the rotation
        # that starts right after the last minimum of the running sum is the
        # only valid one.
        rev = arity[:, ::-1]
        walk = np.cumsum(1 - rev, 1)
        last_min = k - 1 - np.argmin(walk[:, ::-1], 1)
        rot = (last_min[:, None] + 1 + np.arange(k)[None, :]) % k
        arity = np.take_along_axis(rev, rot, 1)[:, ::-1]
        sym = np.where(arity == 2, rng.choice(binary, (m, k)),
                       np.where(arity == 1, rng.choice(unary, (m, k)),
                                np.where(rng.random((m, k)) < 0.5, attr, const)))
        e = np.where(sym == attr, rng.integers(0, ncol, (m, k)).astype(np.float32),
                     np.where(sym == const, rng.uniform(lo, hi, (m, k)).astype(np.float32), 0.0))
        ph[idx, :k] = sym
        ep[idx, :k] = e
    return ph, ep


def _random_target(rng, X, depth=5):
    """A random depth-`depth` expression over the columns of X (float64)."""
    if depth == 0:
        return X[:, rng.integers(X.shape[1])] if rng.random() < 0.7 else np.full(len(X), rng.uniform(-2, 2))
    op = rng.integers(6)
    a = _random_target(rng, X, depth - 1)
    if op == 0:
        return np.sin(a)
    if op == 1:
        return np.exp(np.clip(a, -5, 5))
    if op == 2:
        return np.log(np.abs(a) + 1.0)
    b = _random_target(rng, X, depth - 1)
    if op == 3:
        return a * b
    if op == 4:
        return a / (np.abs(b) + 1.0)
    return a + b


def uneven_batch(seed=11, n_pops=64, pop_range=(256, 30000), rec_range=(100, 1_000_000),
                 feat_range=(1, 32), mean_len=40, len_range=(4, 256), max_size=256, mixed=False):
    """Uneven batch: n_pops populations with log-uniform sizes and record
    counts, 1-32 N(0,1) features, targets from a random depth-5 expression +
    N(0, 0.05) noise, and programs of geometric length (mean 40, 4..256)
    generated as random valid prefix trees.  Returns (grammar, list of
    population dicts with rows / n / phenotype / ephemeral / size).  Every
    population is PDP with the absolute error and the sum; with mixed=True
    each draws its strategy (PP, DP, PDP), error function (absolute or
    squared) and reduction (REDUCEMAX one time in four) instead, from a
    generator of its own, so the programs and datasets stay the same."""
    rng = np.random.default_rng(seed)
    mix = np.random.default_rng(seed + 7919)
    g = G.load(os.path.join(GRAMMARS, "config2_poly.bnf"))
    pops = []
    for p in range(n_pops):
        n = int(np.exp(rng.uniform(np.log(pop_range[0]), np.log(pop_range[1]))))
        nlin = int(np.exp(rng.uniform(np.log(rec_range[0]), np.log(rec_range[1]))))
        nfeat = int(rng.integers(feat_range[0], feat_range[1] + 1))
        X = rng.normal(0.0, 1.0, (nlin, nfeat))
        y = _random_target(rng, X) + rng.normal(0.0, 0.05, nlin)
        rows = np.concatenate([X, y[:, None]], 1).astype(np.float32)
        lengths = np.clip(rng.geometric(1.0 / mean_len, n), len_range[0], len_range[1])
        ph, ep = random_programs(rng, lengths, nfeat, g)
        phf = np.zeros((n, max_size), np.int32)
        epf = np.zeros((n, max_size), np.float32)
        phf[:, :ph.shape[1]] = ph
        epf[:, :ep.shape[1]] = ep
        pop = dict(rows=rows, n=n, phenotype=phf, ephemeral=epf, size=lengths.astype(np.int32),
                   strategy="PDP", error_fn="abs", protected=True, reduce_max=False)
        if mixed:
            pop["strategy"] = ("PP", "DP", "PDP")[int(mix.integers(3))]
            pop["error_fn"] = ("abs", "squared")[int(mix.integers(2))]
            pop["reduce_max"] = bool(mix.random() < 0.25)
        pops.append(pop)
    return g, pops


def default_lanes(strategy, nlin, sm_count=152):
    """The lane count ppi_gpu_set_dataset picks when none is given (the
    reference's rule, accelerator.cc:296-330, on a device of sm_count units)."""
    if strategy == "PP":
        return 1
    if strategy == "PDP":
        return min(nlin, 1024)
    return min(1024, -(-nlin // sm_count))


def adjoint(seed=21, nlin=100_000, population=10_000, max_size=64, mean_len=20):
    """Constant-adjoint configuration: nlin records x 8 N(0,1) features, y = a
    random depth-5 expression (sin/exp/log/*,/) + N(0, 0.05); programs are
    random valid prefix trees over + - * / sin exp log (geometric lengths, mean
    20, 3..max_size) whose leaves are attributes and 1-8 ephemeral constants
    uniform in [-2, 2]; EF squared error, sum.  Returns (grammar, rows,
    phenotype, ephemeral, size)."""
    rng = np.random.default_rng(seed)
    g = G.load(os.path.join(GRAMMARS, "config4_adjoint.bnf"))
    X = rng.normal(0.0, 1.0, (nlin, 8))
    y = _random_target(rng, X) + rng.normal(0.0, 0.05, nlin)
    rows = np.concatenate([X, y[:, None]], 1).astype(np.float32)
    S = g.symbols
    lengths = np.clip(rng.geometric(1.0 / mean_len, population), 3, max_size)
    ph, ep = random_programs(rng, lengths, 8, g, p_unary=0.25)
    attr, const = S["T_ATTRIBUTE"], S["T_CONST"]
    size = lengths.astype(np.int32)
    # exactly k = 1..8 constant leaves (as many as the program has leaves)
    for i in range(population):
        leaves = np.flatnonzero((ph[i, :size[i]] == attr) | (ph[i, :size[i]] == const))
        k = min(len(leaves), int(rng.integers(1, 9)))
        pick = rng.choice(leaves, k, replace=False)
        ph[i, leaves] = attr
        ep[i, leaves] = rng.integers(0, 8, len(leaves)).astype(np.float32)
        ph[i, pick] = const
        ep[i, pick] = rng.uniform(-2.0, 2.0, k).astype(np.float32)
    phf = np.zeros((population, max_size), np.int32)
    epf = np.zeros((population, max_size), np.float32)
    phf[:, :ph.shape[1]] = ph
    epf[:, :ep.shape[1]] = ep
    return g, rows, phf, epf, size
