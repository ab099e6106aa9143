"""PPI's interpreter interface (acc_interpret_init / acc_interpret /
acc_print_time) on the GPU through the adapter, driven the way src/ppi.cc and
src/ppp.cc call it: evolution mode with island callbacks and best index, ppp
test mode and ppp prediction mode.  PARITY math (PPI_GPU_MATH=parity), so the
results must equal the oracle bit for bit."""
import os

import numpy as np
import pytest

from adapter_build import build_driver, run_driver
from helpers import GRAMMARS, assert_bitexact, expected_best, load_golden, oracle_for
from ppi_gpu import grammar as G

pytestmark = pytest.mark.gpu

EF_TEXT = {"abs": "fabs((X)-(Y))", "misclass": "((X)!=(Y))", "squared": "(((X)-(Y))*((X)-(Y)))",
           "cost": "COST[(int)X][(int)Y]"}
CASES = [("cfg2", "PDP", 64), ("cfg1", "PP", 0), ("cfg2max", "DP", 16), ("cfg5", "DP", 40),
         ("allops", "PDP", 0), ("allops_sqmax", "PP", 0)]


def _driver(d, tmp, profiling=False):
    g = G.load(os.path.join(GRAMMARS, d["grammar_file"]))
    cost = None
    if d["ef"] == "cost":
        c = d["cost"]
        cost = "[%d]={%s}" % (c.shape[0], ",".join(
            "{" + ",".join(repr(float(v)) for v in row) + "}" for row in c))
    return build_driver(g, str(tmp), ef=EF_TEXT[d["ef"]], cost=cost, reducemax=bool(d["reduce_max"]),
                        protected=bool(d["protected"]), profiling=profiling)


def _flags(strategy, lanes):
    return ["-strategy", strategy.lower()] + (["-cl-mls", str(lanes)] if lanes else []) + ["-v"]


@pytest.mark.parametrize("name,strategy,lanes", CASES)
def test_evolution_mode(gpu_lib, oracle_lib, tmp_path, name, strategy, lanes):
    d = load_golden(name)
    exe = _driver(d, tmp_path, profiling=(name == "cfg2"))
    rng = np.random.default_rng(5)
    perm = rng.permutation(len(d["size"]))
    gens = [(d["phenotype"], d["ephemeral"], d["size"]),
            (d["phenotype"][perm], d["ephemeral"][perm], d["size"][perm])]
    out, stdout = run_driver(exe, 0, d["rows"], gens, float(d["alpha"]), _flags(strategy, lanes),
                             env={"PPI_GPU_MATH": "parity"})
    nlin = len(d["rows"])
    L = 1 if strategy == "PP" else (lanes if lanes else min(nlin, 1024))
    o = oracle_for(oracle_lib, d)
    for (ph, ep, sz), (fit, best, send_at, recv_at, nimm) in zip(gens, out):
        ref = o.evaluate(ph, ep, sz, strategy, L, float(d["alpha"]))
        assert_bitexact(fit, ref, "%s %s" % (name, strategy))
        # acc_interpret's index: best_individual work-groups sized by the
        # reference's rule for this population, then PickNBest
        assert best == expected_best(oracle_lib, o, ph, ep, sz, strategy, L, float(d["alpha"]))
        assert (send_at, recv_at, nimm) == (0, 1, 0)   # send, then receive, inside the call
    if name == "cfg2":
        assert "gpops_kernel" in stdout and "Device: CUDA" in stdout


def _write_csv(path, rows, header=True):
    """rows as PPI's CSV: '%.9g' round-trips every float32 exactly."""
    with open(path, "w") as f:
        if header:
            f.write(",".join("x%d" % k for k in range(rows.shape[1] - 1)) + ",y\n")
        f.write("# written by the test\n")
        for r in rows:
            f.write(",".join("%.9g" % v for v in r) + "\n")


@pytest.mark.parametrize("name,strategy,lanes", [("cfg2", "PDP", 64), ("cfg5", "DP", 40)])
def test_dataset_read_from_the_csv_file(gpu_lib, oracle_lib, tmp_path, name, strategy, lanes):
    """With PPI's -d flag on the command line the adapter uploads the dataset
    straight from that file (ppi_gpu_set_dataset_csv) instead of main.cc's
    float** rows; the results are the same."""
    d = load_golden(name)
    exe = _driver(d, tmp_path)
    csv = str(tmp_path / "data.csv")
    _write_csv(csv, d["rows"])
    gens = [(d["phenotype"], d["ephemeral"], d["size"])]
    out, stdout = run_driver(exe, 0, d["rows"], gens, float(d["alpha"]),
                             _flags(strategy, lanes) + ["-d", csv], env={"PPI_GPU_MATH": "parity"})
    assert "read from the CSV file" in stdout
    o = oracle_for(oracle_lib, d)
    ref = o.evaluate(*gens[0], strategy, lanes, float(d["alpha"]))
    assert_bitexact(out[0][0], ref, "%s from CSV" % name)
    assert out[0][1] == expected_best(oracle_lib, o, *gens[0], strategy, lanes, float(d["alpha"]))


def test_csv_entry_point_equals_row_upload(gpu_lib, tmp_path):
    d = load_golden("random")
    csv = str(tmp_path / "random.csv")
    _write_csv(csv, d["rows"], header=False)
    import ppi_gpu
    evs = []
    for how in ("csv", "rows"):
        ev = ppi_gpu.Evaluator(d["symtab"], d["max_size"], len(d["size"]), "PDP", 0, d["ef"],
                               d["cost_or_none"], bool(d["reduce_max"]), bool(d["protected"]),
                               "parity")
        if how == "csv":
            assert ev.set_dataset_csv(csv) == d["rows"].shape
        else:
            ev.set_dataset(d["rows"])
        evs.append(ev.evaluate(d["phenotype"], d["ephemeral"], d["size"], 1e-6))
    assert_bitexact(evs[0][0], evs[1][0], "csv vs rows")
    assert evs[0][1] == evs[1][1]
    with pytest.raises(ppi_gpu.PpiGpuError, match="Failed to open dataset file"):
        ev.set_dataset_csv(str(tmp_path / "absent.csv"))


@pytest.mark.parametrize("name,strategy,lanes", CASES[:4])
def test_ppp_modes(gpu_lib, oracle_lib, tmp_path, name, strategy, lanes):
    d = load_golden(name)
    exe = _driver(d, tmp_path)
    o = oracle_for(oracle_lib, d)
    nlin = len(d["rows"])
    L = 1 if strategy == "PP" else (lanes if lanes else min(nlin, 1024))
    for i in d["pred_index"][:3]:
        prog = (d["phenotype"][i:i + 1], d["ephemeral"][i:i + 1], d["size"][i:i + 1])
        (err, *_), = run_driver(exe, 1, d["rows"], [prog], 0.0, _flags(strategy, lanes),
                                env={"PPI_GPU_MATH": "parity"})[0]
        ref = o.evaluate(*prog, strategy, L, 0.0)
        assert_bitexact(err, ref, "ppp test %d" % i)
        (pred, *_), = run_driver(exe, 2, d["rows"], [prog], 0.0, _flags(strategy, lanes),
                                 env={"PPI_GPU_MATH": "parity"})[0]
        assert_bitexact(pred, o.predict(prog[0][0], prog[1][0], prog[2][0]), "ppp predict %d" % i)


def test_init_errors_are_reported_like_the_reference(gpu_lib, tmp_path):
    d = load_golden("cfg2")
    exe = _driver(d, tmp_path)
    prog = (d["phenotype"][:2], d["ephemeral"][:2], d["size"][:2])
    with pytest.raises(RuntimeError, match="Valid strategy"):
        run_driver(exe, 0, d["rows"], [prog], 0.0, ["-strategy", "XYZ"])
    with pytest.raises(RuntimeError, match="compatible type"):
        run_driver(exe, 0, d["rows"], [prog], 0.0, ["-type", "CPU"])
