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
