"""The committed ncu summaries (profiles/*.md): each names the command that
made it, every ncu command leaves the GPU clocks alone
(`--clock-control none`) and runs committed files only, and the launch
lists that bench.py reads its DRAM traffic and issue activity from hold
those figures for every workload the default line reports."""
import glob
import importlib.util
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILES = sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md")))


def _ncu_commands(text):
    """Each ncu command with its continuation lines joined."""
    cmds, cur = [], None
    for line in text.splitlines():
        s = line.strip()
        if cur is not None:
            cur += " " + s.rstrip("\\")
            if not s.endswith("\\"):
                cmds.append(cur)
                cur = None
        elif s.startswith("ncu "):
            if s.endswith("\\"):
                cur = s.rstrip("\\")
            else:
                cmds.append(s)
    return cmds


@pytest.mark.parametrize("path", PROFILES, ids=[os.path.basename(p) for p in PROFILES])
def test_profile_names_its_commands(path):
    text = open(path).read()
    cmds = _ncu_commands(text)
    assert cmds, "no ncu command given"
    for c in cmds:
        assert "--clock-control none" in c, c
        assert "python bench.py" in c, "profiles run the committed bench: " + c
    assert "_work" not in text   # only committed files


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("workload", ["uneven-batch", "uneven-mixed", "stream-4000k-x32-pop30000",
                                      "polynomial-100k-pop30000", "iris-150-pop1000"])
def test_bench_reads_traffic_and_issue_activity(workload):
    b = _bench()
    traffic = b.profile_traffic(workload)
    issue = b.profile_value("launches_" + workload, "issue_active_frac")
    assert traffic is not None and traffic > 0
    assert issue is not None and 0.0 < issue <= 1.0
    # the summary states the same figure it is read from
    text = open(os.path.join(ROOT, "profiles", "launches_%s.md" % workload)).read()
    assert re.search(r"^traffic_bytes_per_step: %d$" % int(traffic), text, re.M)
