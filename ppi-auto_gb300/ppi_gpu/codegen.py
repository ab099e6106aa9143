"""Build-time header generator for the adapter.

PPI's CMake build runs script/read_grammar.py and configure_file to produce,
per grammar and build options, the headers its interpreter compiles against:
``symbol`` (the Symbol enum), ``definitions.h`` (``ERROR(X,Y)``, REDUCEMAX,
PROTECTED, NATIVE) and ``costmatrix`` (``COST``).  The adapter
(ppi-auto_gb300/adapter/accelerator_cuda.cc) additionally needs
``ppi_symbol_map``: the grammar's terminals as ``{Symbol, op, value}`` entries
for ppi_gpu_create.

In PPI's own tree only ``ppi_symbol_map`` is generated here; the other headers
come from PPI's build.  This module can also write equivalents of the three
PPI headers (same macro and enum names, same values) so that the adapter can be
built and tested where PPI's build is not available.

    python3 -m ppi_gpu.codegen -g grammar.bnf -o outdir [--map-only]
        [--ef "fabs((X)-(Y))"] [--cost "[8]={{...}}"] [--reducemax] [--protected] [--native]
"""
from __future__ import annotations

import argparse
import os
import sys

from . import grammar as G

DEFAULT_EF = "fabs((X)-(Y))"
COST_EF = "COST[(int)X][(int)Y]"


def symbol_header(g: G.Grammar) -> str:
    lines = ["/* Symbol enum of the grammar (numbering of script/read_grammar.py). */",
             "#ifndef __SYMBOL_H", "#define __SYMBOL_H", "",
             "#define TERMINAL_MIN %d" % G.TERMINAL_MIN, "#define ATTRIBUTE_MIN %d" % G.ATTRIBUTE_MIN, "",
             "typedef enum {"]
    items = ["NT_%s = %d" % (n, g.symbols["NT_" + n]) for n in g.nonterminals]
    items += ["T_%s = %d" % (n, g.symbols["T_" + n]) for n in g.terminals]
    if g.attributes:
        items.append("T_ATTRIBUTE = %d" % g.t_attribute)
        items += ["T_ATTR%d = %d" % (k, g.symbols["T_ATTR%d" % k]) for k in g.attributes]
    lines.append("   " + ",\n   ".join(items))
    lines.append("} Symbol;")
    if g.t_const is None:
        lines += ["", "#define NOT_USING_T_CONST 1"]
    lines += ["", "#endif", ""]
    return "\n".join(lines)


def definitions_header(ef=None, cost=None, reducemax=False, protected=False, native=False) -> str:
    if ef is None:
        ef = COST_EF if cost else DEFAULT_EF
    out = ["/* Build options of the evaluator (PPI's -DEF / -DREDUCEMAX / -DPROTECTED / -DNATIVE). */",
           "#define ERROR(X,Y) %s" % ef]
    for name, on in (("REDUCEMAX", reducemax), ("PROTECTED", protected), ("NATIVE", native)):
        out.append(("#define %s 1" % name) if on else ("/* #undef %s */" % name))
    return "\n".join(out) + "\n"


def costmatrix_header(cost=None) -> str:
    return ("const float COST[]%s;\n" % cost) if cost else "\n"


def write(g: G.Grammar, outdir, map_only=False, **opts):
    os.makedirs(outdir, exist_ok=True)
    files = {"ppi_symbol_map": G.symbol_map_header(g)}
    if not map_only:
        files["symbol"] = symbol_header(g)
        files["definitions.h"] = definitions_header(**opts)
        files["costmatrix"] = costmatrix_header(opts.get("cost"))
    for name, text in files.items():
        with open(os.path.join(outdir, name), "w") as f:
            f.write(text)
    return sorted(files)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("-g", "--grammar", required=True)
    ap.add_argument("-o", "--output-dir", required=True)
    ap.add_argument("--map-only", action="store_true")
    ap.add_argument("--ef")
    ap.add_argument("--cost")
    ap.add_argument("--reducemax", action="store_true")
    ap.add_argument("--protected", action="store_true")
    ap.add_argument("--native", action="store_true")
    a = ap.parse_args(argv)
    g = G.load(a.grammar)
    names = write(g, a.output_dir, a.map_only, ef=a.ef, cost=a.cost, reducemax=a.reducemax,
                  protected=a.protected, native=a.native)
    print("wrote", ", ".join(names), "to", a.output_dir)
    return 0


if __name__ == "__main__":
    sys.exit(main())
