"""BNF grammar reader: Symbol numbering, rule tables and the Symbol -> op map.

PPI numbers its grammar symbols at build time with script/read_grammar.py and
the generated ``symbol`` / ``grammar`` headers.  This module restates that
numbering so the GPU evaluator and decoder can be driven from the same BNF:

* non-terminals are numbered from 0: ``NT_INICIAL`` first (the ``S =`` line),
  then every left-hand side in order of definition
  (script/read_grammar.py:78-106);
* terminals are numbered from ``TERMINAL_MIN`` = 10000 in order of first
  appearance on a right-hand side, operators renamed by
  ``interpreter()`` (script/read_grammar.py:19-41, 132-194, 275);
* a terminal whose name contains ``ATTR`` is an attribute: the first one
  adds ``T_ATTRIBUTE`` right after the last ordinary terminal, and
  ``T_ATTRk`` = ``ATTRIBUTE_MIN`` + k with ``ATTRIBUTE_MIN`` = 20000
  (script/read_grammar.py:146-152, 276);
* the rule tables ``gramatica[nt][k]`` / ``tamanhos[nt]`` list the
  alternatives of each non-terminal in order (script/read_grammar.py:78-130,
  207-229); ``MAX_QUANT_SIMBOLOS_POR_REGRA`` is the longest alternative.

The op map assigns each terminal its evaluator op (the ``case T_X:`` blocks of
src/interpreter/interpreter_core and ``T_ATTRIBUTE`` / ``T_CONST`` of
src/interpreter/accelerator.cl:37-51); named constants become literals with the
float value the interpreter pushes (interpreter_core:152-793).
"""
from __future__ import annotations

import dataclasses
import numpy as np

TERMINAL_MIN = 10000
ATTRIBUTE_MIN = 20000

# Evaluator op codes; must match enum ppi_op in include/ppi_gpu.h.
OPS = [
    "INVALID", "ATTRIBUTE", "CONST", "LITERAL",
    # ternary
    "IF_THEN_ELSE",
    # binary
    "AND", "OR", "XOR", "GREATER", "GREATEREQUAL", "LESS", "LESSEQUAL", "EQUAL",
    "NOTEQUAL", "ADD", "SUB", "MULT", "MEAN", "MAX", "MIN", "MOD", "POW", "DIV",
    # unary
    "NOT", "ABS", "POW2", "POW3", "POW4", "POW5", "NEG", "ROUND", "CEIL", "FLOOR",
    "EXP", "EXP10", "EXP2", "SIN", "COS", "STEP", "SIGN", "LOGISTIC", "GAMMA",
    "GAUSS", "SQRT", "LOG", "LOG10", "LOG2", "TAN",
]
OP = {name: i for i, name in enumerate(OPS)}
TERNARY = {"IF_THEN_ELSE"}
BINARY = set(OPS[5:23])
UNARY = set(OPS[23:])


def op_arity(op: int) -> int:
    name = OPS[op]
    if name in TERNARY:
        return 3
    if name in BINARY:
        return 2
    if name in UNARY:
        return 1
    return 0


# Float constants of the generated symbol header (script/read_grammar.py:235-273),
# as the float literals the interpreter pushes.
NAMED_CONSTANTS = {
    "PI": "3.14159274101257", "PI_2": "1.57079637050629", "PI_4": "0.78539818525314",
    "1_PI": "0.31830987334251", "2_PI": "0.63661974668503",
    "2_SQRTPI": "1.12837922573090", "SQRT2": "1.41421353816986",
    "SQRT1_2": "0.70710676908493", "E": "2.71828174591064", "LOG2E": "1.44269502162933",
    "LOG10E": "0.43429449200630", "LN2": "0.69314718246460", "LN10": "2.30258512496948",
}
for _k in range(0, 101):
    NAMED_CONSTANTS[str(_k)] = f"{_k}.0"
for _k in range(1, 101):
    NAMED_CONSTANTS[f"N{_k}"] = f"-{_k}.0"

_OPERATOR_NAMES = {">": "GREATER", ">=": "GREATEREQUAL", "<": "LESS", "<=": "LESSEQUAL",
                   "=": "EQUAL", "!=": "NOTEQUAL", "+": "ADD", "-": "SUB", "*": "MULT",
                   "/": "DIV"}


def terminal_name(token: str) -> str:
    """Enum name (without ``T_``) of a grammar terminal token."""
    if token in _OPERATOR_NAMES:
        return _OPERATOR_NAMES[token]
    return token.upper()


def _is_nonterminal(tok: str) -> bool:
    return len(tok) >= 2 and tok[0] == "<" and tok[-1] == ">"


def _nt_name(tok: str) -> str:
    return tok[1:-1].upper()


@dataclasses.dataclass
class Grammar:
    nonterminals: list            # NT names in enum order ("INICIAL" first)
    terminals: list               # T_ names (without T_) of ordinary terminals in enum order
    attributes: list              # attribute indices k of T_ATTRk, in order of appearance
    rules: list                   # rules[nt] = list of alternatives (lists of Symbol values)
    symbols: dict                 # enum name (NT_X / T_X) -> Symbol value
    max_rule: int                 # MAX_QUANT_SIMBOLOS_POR_REGRA

    @property
    def t_attribute(self):
        return self.symbols.get("T_ATTRIBUTE")

    @property
    def t_const(self):
        return self.symbols.get("T_CONST")

    def symbol_table(self):
        """(symbol, op, value) entries for every terminal the evaluator can meet."""
        out = []
        for name in self.terminals:
            v = self.symbols["T_" + name]
            if name == "CONST":
                out.append((v, OP["CONST"], 0.0))
            elif name in NAMED_CONSTANTS:
                out.append((v, OP["LITERAL"], float(np.float32(NAMED_CONSTANTS[name]))))
            elif name in OP and OP[name] >= OP["IF_THEN_ELSE"]:
                out.append((v, OP[name], 0.0))
            else:
                out.append((v, OP["INVALID"], 0.0))
        if self.t_attribute is not None:
            out.append((self.t_attribute, OP["ATTRIBUTE"], 0.0))
        return out

    def symbol_table_arrays(self):
        t = self.symbol_table()
        return (np.array([e[0] for e in t], np.int32), np.array([e[1] for e in t], np.int32),
                np.array([e[2] for e in t], np.float32))

    def decode_tables(self):
        """Flat rule tables for the decoders.

        Returns (rule_first[nt], rule_count[nt], alt_len[a], alt_syms[a, max_rule]) where
        alternative a = rule_first[nt] + k is gramatica[nt][k].
        """
        first, count, lens, syms = [], [], [], []
        for alts in self.rules:
            first.append(len(lens))
            count.append(len(alts))
            for alt in alts:
                lens.append(len(alt))
                syms.append(list(alt) + [0] * (self.max_rule - len(alt)))
        return (np.array(first, np.int32), np.array(count, np.int32), np.array(lens, np.int32),
                np.array(syms, np.int32).reshape(-1, self.max_rule))

    def symbol_header_enum(self) -> str:
        """The enum body of the generated ``symbol`` header (for comparisons)."""
        parts = ["NT_" + n for n in self.nonterminals]
        parts += ["T_" + n for n in self.terminals]
        if self.attributes:
            parts += ["T_ATTRIBUTE"] + ["T_ATTR%d" % k for k in self.attributes]
        return ", ".join(parts)


def parse_bnf(text: str) -> Grammar:
    tokens = []
    for line in text.splitlines():
        if line.lstrip().startswith("#"):
            continue
        tokens += line.split()
    if "S" not in tokens or "P" not in tokens:
        raise ValueError("grammar needs an 'S =' start line and a 'P =' production list")
    s = tokens.index("S")
    p = tokens.index("P")
    start = [t for t in tokens[s + 1:p] if _is_nonterminal(t)]
    if not start:
        raise ValueError("empty start rule")
    # Productions: '<lhs> ::= alt | alt ...'
    prods = []   # (lhs, [alternatives as token lists])
    body = tokens[p + 1:]
    i = 0
    while i < len(body):
        if i + 1 < len(body) and body[i + 1] == "::=":
            lhs = body[i]
            if not _is_nonterminal(lhs):
                raise ValueError("left-hand side must be a <non-terminal>: %r" % lhs)
            i += 2
            alts, cur = [], []
            while i < len(body) and not (i + 1 < len(body) and body[i + 1] == "::="):
                if body[i] == "|":
                    alts.append(cur)
                    cur = []
                else:
                    cur.append(body[i])
                i += 1
            alts.append(cur)
            if any(len(a) == 0 for a in alts):
                raise ValueError("empty alternative in rule %s" % lhs)
            prods.append((lhs, alts))
        else:
            i += 1
    nts = ["INICIAL"]
    for lhs, _ in prods:
        n = _nt_name(lhs)
        if n in nts:
            raise ValueError("non-terminal %s defined twice" % lhs)
        nts.append(n)
    symbols = {"NT_" + n: k for k, n in enumerate(nts)}
    terminals, attributes = [], []
    for _, alts in prods:
        for alt in alts:
            for tok in alt:
                if _is_nonterminal(tok):
                    continue
                name = terminal_name(tok)
                if "ATTR" in tok.upper():
                    k = int(tok[4:])
                    if k not in attributes:
                        attributes.append(k)
                elif name not in terminals:
                    terminals.append(name)
    for k, name in enumerate(terminals):
        symbols["T_" + name] = TERMINAL_MIN + k
    if attributes:
        symbols["T_ATTRIBUTE"] = TERMINAL_MIN + len(terminals)
        for k in attributes:
            symbols["T_ATTR%d" % k] = ATTRIBUTE_MIN + k

    def sym(tok):
        if _is_nonterminal(tok):
            n = _nt_name(tok)
            if "NT_" + n not in symbols:
                raise ValueError("undefined non-terminal %s" % tok)
            return symbols["NT_" + n]
        if "ATTR" in tok.upper():
            return ATTRIBUTE_MIN + int(tok[4:])
        return symbols["T_" + terminal_name(tok)]

    rules = [[[sym(t) for t in start]]]
    for _, alts in prods:
        rules.append([[sym(t) for t in alt] for alt in alts])
    max_rule = max(len(a) for alts in rules for a in alts)
    return Grammar(nts, terminals, attributes, rules, symbols, max_rule)


def load(path) -> Grammar:
    with open(path) as f:
        return parse_bnf(f.read())


def max_phenotype_size(g: Grammar, number_of_bits: int, bits_per_gene: int, mps: int) -> int:
    """max_size_phenotype of src/ppi.cc:307."""
    return min(g.max_rule * number_of_bits // bits_per_gene, mps)


def effective_bits_per_gene(g: Grammar, bits_per_gene: int) -> int:
    """-bg raised until every rule list fits (src/ppi.cc:263-270)."""
    import math
    bg = bits_per_gene
    for alts in g.rules:
        need = math.ceil(math.log10(len(alts)) / math.log10(2.0))
        bg = max(bg, need)
    return bg


def symbol_map_header(g: Grammar, guard="PPI_SYMBOL_MAP") -> str:
    """C header listing {Symbol, op, value} for the adapter.

    The entries name the enum constants of the generated ``symbol`` header, so
    their values always come from the reference build itself.
    """
    lines = ["/* Generated by ppi_gpu.grammar.symbol_map_header: Symbol -> evaluator op. */",
             "#ifndef %s" % guard, "#define %s" % guard,
             "static const ppi_symbol_entry ppi_symbol_map[] = {"]
    t = g.symbol_table()
    names = {v: k for k, v in g.symbols.items()}
    for sym, op, val in t:
        lit = float(np.float32(val)).hex() + "f"      # exact: hexadecimal float literal
        lines.append("   { %s, PPI_OP_%s, %s }," % (names[sym], OPS[op], lit))
    lines += ["};", "#endif", ""]
    return "\n".join(lines)
