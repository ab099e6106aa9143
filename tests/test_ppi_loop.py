"""PPI's own evolution loop (the reference's unchanged src/main.cc, src/ppi.cc,
src/ppp.cc, common, server, client, util and sequential interpreter) linked
with the GB300 adapter in place of src/interpreter/accelerator.cc, with
test-only Poco stand-ins (tests/integration/poco_stub).  Needs the reference
tree, so it runs where the oracle's reference build was made; on a machine
without a GPU the accelerated run must fail the way PPI reports a failed
accelerator (init message, then exit code 8 from main's std::exception
handler, src/main.cc:201-203)."""
import os
import subprocess

import pytest

from oracle.build_ref import reference_root

REF_SRC = os.path.join(reference_root(), "src")
DATA = os.path.join(reference_root(), "problem", "polynomial", "data.csv")


@pytest.fixture(scope="module")
def ppi_exe(tmp_path_factory):
    from oracle import pyoracle
    from ppi_gpu import grammar as G
    from adapter_build import build_ppi
    man = pyoracle.ref_manifest()
    if not man or not os.path.exists(os.path.join(REF_SRC, "ppi.cc")) or not os.path.exists(DATA):
        pytest.skip("reference tree not present")
    info = man["polynomial"]
    generated = os.path.join(pyoracle.REF, "polynomial", "include")
    return build_ppi(REF_SRC, generated, G.load(info["grammar"]), str(tmp_path_factory.mktemp("ppi")))


def _run(exe, *flags):
    return subprocess.run([exe, "-d", DATA, "-port", "9999", "-g", "4", "-ps", "64", "-s", "1", "-e"] +
                          list(flags), capture_output=True, text=True, timeout=120)


def test_ppi_evolution_loop_runs(ppi_exe):
    r = _run(ppi_exe)
    assert r.returncode == 0, r.stderr
    assert "> Overall best:" in r.stdout


def test_ppi_accelerated_run_goes_through_the_adapter(ppi_exe):
    torch = pytest.importorskip("torch")
    r = _run(ppi_exe, "-acc")
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stderr
        assert "> Overall best:" in r.stdout
    else:
        assert "Error in initialization phase." in r.stderr
        assert r.returncode == 8
