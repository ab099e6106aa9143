#!/usr/bin/env python3
"""Generate golden vectors from the reference's own code (oracle/_ref).

Run after ``python3 oracle/build_ref.py`` in a checkout that has the reference
tree.  For every reference configuration built there (grammar x EF x COST x
REDUCEMAX x PROTECTED) this script draws seeded genomes and a seeded synthetic
dataset shaped like the configuration's problem, and records what the
reference computes:

* decode (src/ppi.cc:106-182): phenotype / ephemeral / size / bits consumed;
* sequential interpreter (src/interpreter/sequential.cc): fitness with
  alpha = 1e-6, best index, and per-record predictions of a few programs;
* the OpenCL kernels (src/interpreter/accelerator.cl via oracle/cl_shim.h)
  for PP, PDP and DP at two lane counts each: fitness and best index.

Output: tests/golden/<config>.npz (compressed).  The datasets are synthetic
(no reference data file is copied).
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "ppi-auto_gb300"))
sys.path.insert(0, REPO)

from ppi_gpu import grammar as G  # noqa: E402
from oracle import pyoracle as P  # noqa: E402

EF_KIND = {"((X)!=(Y))": "misclass", "fabs((X)-(Y))": "abs",
           "(((X)-(Y))*((X)-(Y)))": "squared", "ppi_guarded_cost_(COST, X, Y)": "cost"}
ALPHA = np.float32(1e-6)
STRATS = [("PP", 16), ("PDP", 64), ("PDP", 7), ("DP", 32), ("DP", 5)]


def cost_matrix(text):
    if not text:
        return None
    rows = re.findall(r"\{([^{}]*)\}", text)
    return np.array([[float(x) for x in r.split(",")] for r in rows], np.float32)


def dataset(name, g, ef, rng):
    nfeat = (max(g.attributes) + 1) if g.attributes else 1
    nlin = {"iris": 150, "cfg1": 150, "polynomial": 20}.get(name, 301)
    if name in ("iris", "cfg1"):
        lo = np.array([4, 2, 1, 0.1], np.float32)
        hi = np.array([8, 4.5, 7, 2.5], np.float32)
        X = (lo + (hi - lo) * rng.random((nlin, 4))).astype(np.float32)
    elif name == "polynomial":
        X = np.linspace(-1, 0.9, nlin, dtype=np.float32)[:, None]
    else:
        X = rng.normal(0, 1.5, (nlin, nfeat)).astype(np.float32)
    if ef == "misclass":
        y = rng.integers(0, 3, nlin).astype(np.float32)
    elif ef == "cost":
        y = rng.integers(0, 8, nlin).astype(np.float32)
    else:
        y = (X[:, 0] ** 2 - X[:, -1] + rng.normal(0, 0.1, nlin)).astype(np.float32)
    return np.concatenate([X, y[:, None]], 1).astype(np.float32)


def make(name, info, seed):
    rng = np.random.default_rng(seed)
    g = G.load(info["grammar"])
    ref = P.RefBuild(name)
    mps = ref.max_size
    nb, bc = 2000, 16
    bg = G.effective_bits_per_gene(g, 8)
    pop = 96
    genomes = rng.integers(0, 2, (pop, nb), dtype=np.uint8)
    rph, rep, rsz, ral = ref.decode(genomes, bg, bc, -10.0, 10.0, mps)
    over = rsz > mps
    ph = np.zeros((pop, mps), np.int32)
    ep = np.zeros((pop, mps), np.float32)
    sz = rsz.copy()
    sz[over] = 0
    for i in range(pop):
        if sz[i] > 0:
            ph[i, :sz[i]] = rph[i, :sz[i]]
            ep[i, :sz[i]] = rep[i, :sz[i]]
    # a few hand-made edge rows: size 0 and a lone terminal
    sz[5] = 0
    ef = EF_KIND[info["ef"]]
    rows = dataset(name, g, ef, rng)
    out = dict(genomes=np.packbits(genomes, axis=1), nb=nb, bg=bg, bc=bc, lo=-10.0, hi=10.0,
               max_size=mps, ref_size=rsz, ref_allele=ral, phenotype=ph, ephemeral=ep, size=sz,
               rows=rows, alpha=ALPHA, ef=ef, cost=cost_matrix(info["cost"]) if info["cost"] else
               np.zeros((0, 0), np.float32), reduce_max=info["reduce_max"],
               protected=info["protected"], symbol_enum=info["symbol_enum"],
               grammar_file=os.path.basename(info["grammar"]))
    first, count, alen, asyms = g.decode_tables()
    sv, so, sl = g.symbol_table_arrays()
    out.update(rule_first=first, rule_count=count, alt_len=alen, alt_syms=asyms,
               max_rule=g.max_rule, t_const=g.t_const if g.t_const is not None else -1,
               t_attribute=g.t_attribute if g.t_attribute is not None else -1,
               sym_values=sv, sym_ops=so, sym_literals=sl)
    fit, best = ref.seq_evaluate(rows, ph, ep, sz, alpha=float(ALPHA))
    out["seq_fitness"], out["seq_best"] = fit, best
    valid = [i for i in range(pop) if sz[i] > 0][:6]
    preds = []
    for i in valid:
        p_, _ = ref.seq_evaluate(rows, ph[i:i + 1], ep[i:i + 1], sz[i:i + 1], prediction=True)
        preds.append(p_)
    out["pred_index"] = np.array(valid, np.int32)
    out["seq_pred"] = np.array(preds, np.float32)
    for strat, L in STRATS:
        f, b = ref.cl_evaluate(strat, rows, ph, ep, sz, L, 16, alpha=float(ALPHA))
        out["cl_%s_%d_fitness" % (strat, L)] = f
        out["cl_%s_%d_best" % (strat, L)] = b
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return name, int((sz > 0).sum()), int(over.sum())


def main():
    man = P.ref_manifest()
    if not man:
        print("oracle/_ref not built: run python3 oracle/build_ref.py first")
        return 1
    for k, (name, info) in enumerate(sorted(man.items())):
        print(make(name, info, 1000 + k))
    return 0


if __name__ == "__main__":
    sys.exit(main())
