"""bench.py's reference arm (CPU only): the JSON line it prints for a
single-population workload and for the mixed-settings batch, and the
`unavailable` line for the workload the reference has no counterpart of."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"] + list(args),
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_reference_arm_line_iris():
    d = _run("--workload", "iris", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("iris")


def test_reference_arm_adjoint_is_unavailable():
    d = _run("--workload", "adjoint", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and "unavailable" in d


def test_reference_arm_mixed_batch_names_its_workload():
    """The mixed-settings batch (strategy, error function and reduction drawn
    per population) on the CPU: the same populations as the GPU arm's
    `uneven-mixed` workload, named so."""
    d = _run("--workload", "uneven-mixed", "--steps", "1", "--warmup", "0", "--cpu-fraction", "0.001")
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["config"]["workload"].endswith("-mixed")
    assert d["cpu_baseline"]["kind"] == "port"
