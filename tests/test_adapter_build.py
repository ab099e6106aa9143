"""The adapter (acc_interpret_* over the C ABI) compiles as a drop-in: against
generated equivalents of PPI's headers and, where the reference tree is
present, against PPI's own accelerator.h and read_grammar.py output.  Nothing
here runs on a GPU."""
import os

import pytest

from adapter_build import build_driver
from helpers import GRAMMARS
from ppi_gpu import grammar as G


@pytest.mark.parametrize("opts", [dict(), dict(ef="((X)!=(Y))", protected=True),
                                  dict(cost="[3]={{0,1,2},{1,0,1},{2,1,0}}", profiling=True),
                                  dict(reducemax=True, native=True)])
def test_adapter_compiles_with_generated_headers(tmp_path, opts):
    g = G.load(os.path.join(GRAMMARS, "config2_poly.bnf"))
    exe = build_driver(g, str(tmp_path), **opts)
    assert os.path.exists(exe)


def test_adapter_compiles_against_ppi_headers(tmp_path):
    from oracle import pyoracle
    man = pyoracle.ref_manifest()
    from oracle.build_ref import reference_root
    ref_interp = os.path.join(reference_root(), "src", "interpreter")
    if not man or not os.path.exists(os.path.join(ref_interp, "accelerator.h")):
        pytest.skip("reference tree not present")
    for name in ("cfg2", "iris", "random"):
        info = man[name]
        g = G.load(info["grammar"])
        inc = os.path.join(pyoracle.REF, name, "include")
        exe = build_driver(g, str(tmp_path / name), ppi_headers=(ref_interp, inc))
        assert os.path.exists(exe)
