"""Grammar reader: Symbol numbering and rule tables against the reference's
generated headers (script/read_grammar.py output recorded in the fixtures)."""
import os

import numpy as np
import pytest

from helpers import GRAMMARS, enum_values, golden_names, load_golden
from ppi_gpu import grammar as G


@pytest.mark.parametrize("name", golden_names())
def test_symbol_numbering_matches_reference_header(name):
    d = load_golden(name)
    ref = enum_values(d["symbol_enum"])
    path = os.path.join(GRAMMARS, d["grammar_file"])
    if os.path.exists(path):
        g = G.load(path)
        assert g.symbols == ref
        first, count, alen, asyms = g.decode_tables()
        np.testing.assert_array_equal(first, d["rule_first"])
        np.testing.assert_array_equal(asyms, d["alt_syms"])
    # the table stored in the fixture covers every terminal of the enum
    names = {v: k for k, v in ref.items()}
    for sym in d["sym_values"]:
        assert names[int(sym)].startswith("T_")


def test_reference_grammars_live():
    from oracle import pyoracle
    man = pyoracle.ref_manifest()
    if not man:
        pytest.skip("reference not built here")
    for name, info in man.items():
        g = G.load(info["grammar"])
        assert g.symbols == enum_values(info["symbol_enum"]), name
        assert ("T_CONST" not in g.symbols) == info["not_using_t_const"]


def test_operator_names_and_ops():
    g = G.parse_bnf("S = <e>\nP = <e> ::= + <e> <e> | >= <e> <e> | pi | N3 | attr2 | const | zz\n")
    assert [t for t in g.terminals] == ["ADD", "GREATEREQUAL", "PI", "N3", "CONST", "ZZ"]
    assert g.symbols["T_ADD"] == 10000 and g.symbols["T_ATTRIBUTE"] == 10006
    assert g.symbols["T_ATTR2"] == 20002
    table = {s: (op, v) for s, op, v in g.symbol_table()}
    assert table[g.symbols["T_PI"]] == (G.OP["LITERAL"], float(np.float32(3.14159274101257)))
    assert table[g.symbols["T_N3"]] == (G.OP["LITERAL"], -3.0)
    assert table[g.symbols["T_ZZ"]][0] == G.OP["INVALID"]
    assert table[g.symbols["T_ATTRIBUTE"]][0] == G.OP["ATTRIBUTE"]


def test_grammar_errors():
    with pytest.raises(ValueError):
        G.parse_bnf("P = <e> ::= x")
    with pytest.raises(ValueError):
        G.parse_bnf("S = <e>\nP = <e> ::= <f>")
    with pytest.raises(ValueError):
        G.parse_bnf("S = <e>\nP = <e> ::= x\n <e> ::= y")


def test_max_phenotype_size_and_bits_per_gene():
    g = G.load(os.path.join(GRAMMARS, "config2_poly.bnf"))
    assert G.max_phenotype_size(g, 4000, 8, 128) == 128
    big = G.parse_bnf("S = <e>\nP = <e> ::= " + " | ".join("attr%d" % k for k in range(300)))
    assert G.effective_bits_per_gene(big, 8) == 9


def test_symbol_map_header_lists_every_terminal():
    g = G.load(os.path.join(GRAMMARS, "config2_poly.bnf"))
    h = G.symbol_map_header(g)
    for name in g.terminals:
        assert "T_%s," % name in h
    assert "T_ATTRIBUTE, PPI_OP_ATTRIBUTE" in h
