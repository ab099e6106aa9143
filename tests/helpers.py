"""Shared helpers of the test suite: golden fixtures, the oracle built from a
fixture's configuration, and program generators."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GRAMMARS = os.path.join(os.path.dirname(GOLDEN), "..", "ppi-auto_gb300", "grammars")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    d = {k: z[k] for k in z.files}
    for k in ("ef", "symbol_enum", "grammar_file"):
        d[k] = str(d[k])
    for k in ("nb", "bg", "bc", "max_size", "max_rule", "t_const", "t_attribute", "reduce_max",
              "protected", "seq_best"):
        d[k] = int(d[k])
    d["genomes_bits"] = np.unpackbits(d["genomes"], axis=1)[:, :d["nb"]]
    d["symtab"] = (d["sym_values"], d["sym_ops"], d["sym_literals"])
    d["cost_or_none"] = d["cost"] if d["cost"].size else None
    return d


def oracle_for(pyoracle, d, float_math=False, rows=None):
    return pyoracle.Oracle(d["rows"] if rows is None else rows, d["symtab"], d["ef"],
                           d["cost_or_none"], d["reduce_max"], d["protected"], float_math)


class Tables:
    """Grammar-table view of a fixture, shaped like ppi_gpu.grammar.Grammar."""

    def __init__(self, d):
        self.d = d
        self.max_rule = d["max_rule"]
        self.t_const = d["t_const"] if d["t_const"] >= 0 else None
        self.t_attribute = d["t_attribute"] if d["t_attribute"] >= 0 else None

    def decode_tables(self):
        return (self.d["rule_first"], self.d["rule_count"], self.d["alt_len"], self.d["alt_syms"])


def enum_values(text):
    """Values of a C enum body such as the generated `symbol` header's."""
    out, nxt = {}, 0
    env = {"TERMINAL_MIN": 10000, "ATTRIBUTE_MIN": 20000}
    for part in text.split(","):
        part = part.strip()
        if not part:
            continue
        if "=" in part:
            name, expr = [s.strip() for s in part.split("=", 1)]
            val = eval(expr, {}, env)
        else:
            name, val = part, nxt
        out[name] = val
        nxt = val + 1
    return out


def device_sm_count():
    """Compute units the library's automatic best_individual group size uses."""
    import torch
    return torch.cuda.get_device_properties(0).multi_processor_count


def auto_best_group(population):
    """The reference's best_individual work-group size for a population on
    this device: min(1024, ceil(population / compute units))
    (src/interpreter/accelerator.cc:348)."""
    cu = device_sm_count()
    return max(1, min(1024, -(-int(population) // cu)))


def expected_best(oracle_lib, o, ph, ep, sz, strategy, lanes, alpha, rule="accelerator",
                  group=None, population=None):
    """The best index the reference returns for these programs.

    sequential: util::PickNBest over the alpha-included fitness
    (sequential.cc:203).  accelerator: best_individual over work-groups of
    `group` programs (default: the automatic size for `population`, itself
    defaulting to the number of programs), then PickNBest over the group
    winners, comparing error/nlin for PP/PDP and the alpha-included fitness for
    DP (accelerator.cc:491,500,848-849,871-880)."""
    fit = o.evaluate(ph, ep, sz, strategy, lanes, alpha)
    if rule == "sequential":
        return oracle_lib.best_index(fit)
    vals = fit if strategy == "DP" else o.evaluate(ph, ep, sz, strategy, lanes, 0.0)
    if group is None or group <= 0:
        group = auto_best_group(population or len(sz))
    return oracle_lib.best_index_accelerator(vals, group)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.int32)


def assert_bitexact(a, b, what=""):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    same = (bits(a) == bits(b)) | (np.isnan(a) & np.isnan(b))
    if not same.all():
        i = np.flatnonzero(~same)[:5]
        raise AssertionError("%s: %d of %d differ, e.g. idx %s: %s vs %s" % (
            what, (~same).sum(), a.size, i.tolist(), a.ravel()[i].tolist(), b.ravel()[i].tolist()))


def make_evaluator(d, strategy="PDP", lanes=0, math="parity", population=None, max_size=None,
                   rows=None, best_rule="accelerator", best_group=0):
    import ppi_gpu
    ev = ppi_gpu.Evaluator(d["symtab"], max_size or d["max_size"],
                           population or len(d["size"]), strategy, lanes, d["ef"],
                           d["cost_or_none"], bool(d["reduce_max"]), bool(d["protected"]), math,
                           best_rule=best_rule, best_group=best_group)
    ev.set_dataset(d["rows"] if rows is None else rows)
    return ev


class ProgramGen:
    """Random well-formed (or deliberately malformed) prefix programs over a
    fixture's symbol table, as phenotype / ephemeral rows."""

    def __init__(self, d, rng, ncol):
        from ppi_gpu import grammar as G
        self.G = G
        self.rng = rng
        self.ncol = ncol
        self.by_op = {}
        for s, op in zip(d["sym_values"], d["sym_ops"]):
            self.by_op.setdefault(int(op), []).append(int(s))
        ops = list(self.by_op)
        self.un = [o for o in ops if G.op_arity(o) == 1]
        self.bi = [o for o in ops if G.op_arity(o) == 2]
        self.ter = [o for o in ops if G.op_arity(o) == 3]
        self.leaf = [o for o in ops if G.op_arity(o) == 0]

    def leaf_tok(self):
        op = self.leaf[self.rng.integers(len(self.leaf))]
        sym = self.by_op[op][self.rng.integers(len(self.by_op[op]))]
        if op == self.G.OP["ATTRIBUTE"]:
            return sym, float(self.rng.integers(self.ncol - 1))
        if op == self.G.OP["CONST"]:
            return sym, float(np.float32(self.rng.uniform(-10, 10)))
        return sym, 0.0

    def op_tok(self, arity):
        pool = {1: self.un, 2: self.bi, 3: self.ter}[arity]
        op = pool[self.rng.integers(len(pool))]
        return self.by_op[op][0], 0.0

    def random(self, n_internal, p_un=0.3, p_ter=0.05):
        """Random tree with about n_internal operator nodes (prefix order)."""
        def build(k):
            if k <= 0:
                return [self.leaf_tok()]
            u = self.rng.random()
            if self.ter and u < p_ter and k >= 3:
                a = self.rng.integers(0, k - 1)
                b = self.rng.integers(0, k - 1 - a)
                return [self.op_tok(3)] + build(a) + build(b) + build(k - 1 - a - b)
            if self.un and u < p_ter + p_un:
                return [self.op_tok(1)] + build(k - 1)
            a = self.rng.integers(0, k)
            return [self.op_tok(2)] + build(a) + build(k - 1 - a)
        return build(n_internal)

    def full(self, depth):
        """Complete binary tree of the given depth (register need depth-1)."""
        if depth == 0:
            return [self.leaf_tok()]
        return [self.op_tok(2)] + self.full(depth - 1) + self.full(depth - 1)

    @staticmethod
    def rows(programs, max_size):
        n = len(programs)
        ph = np.zeros((n, max_size), np.int32)
        ep = np.zeros((n, max_size), np.float32)
        sz = np.zeros(n, np.int32)
        for i, p in enumerate(programs):
            p = p[:max_size]
            sz[i] = len(p)
            for k, (s, e) in enumerate(p):
                ph[i, k] = s
                ep[i, k] = e
        return ph, ep, sz
