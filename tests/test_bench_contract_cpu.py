"""The reference arm of bench.py runs on CPU: its JSON line keeps the contract."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1",
                          "--scale", "0.002"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1 and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["config"]["persons"] > 10_000 and "workload" in d["config"]
    assert d["days_simulated"] == 100 and d["days_per_step"] == 50


def test_parity_helpers_flag_a_planted_difference():
    # the comparisons bench.py reports: equal records pass, one changed field fails
    sys.path.insert(0, ROOT)
    sys.path.insert(0, ROOT)
    import bench
    import numpy as np
    rows = [{"rc": 0, "counts": list(range(16)), "infected": 5, "rand_offset": 100 + d} for d in range(3)]
    state = {k: np.arange(10, dtype=np.uint8) for k in bench.STATE_FIELDS}
    rec = {"rows": rows, "digests": bench.state_digests(state)}
    same = bench.parity_vs_oracle(rec, json.loads(json.dumps(rec)))
    assert same["equal"] and same["days"] == 3
    planted = json.loads(json.dumps(rec))
    planted["rows"][1]["rand_offset"] += 1
    bad = bench.parity_vs_oracle(rec, planted)
    assert not bad["equal"] and bad["mismatches"] == ["day 1 rand_offset"]
    state2 = dict(state, gen_s=state["gen_s"].copy())
    state2["gen_s"][3] ^= 1
    bad = bench.parity_vs_oracle(rec, {"rows": rows, "digests": bench.state_digests(state2)})
    assert bad["mismatches"] == ["final gen_s"]


def test_tuning_spec_sets_named_launch_shapes_and_rejects_unknown_ones():
    sys.path.insert(0, ROOT)
    import bench

    class Engine:
        def __init__(self):
            self.t = {"infect_coop": 0, "sched_tf": 0, "radix_threads": 256}
            self.tuned = False

        def tuning(self):
            return dict(self.t)

        def set_tuning(self, t):
            self.t = dict(t)

        def autotune(self):
            self.tuned = True
            return dict(self.t)

    e = Engine()
    assert bench.apply_tuning(e, "sched_tf=1,infect_coop=1") == {"infect_coop": 1, "sched_tf": 1, "radix_threads": 256}
    assert not e.tuned
    bench.apply_tuning(e, "auto")
    assert e.tuned
    with pytest.raises(SystemExit):
        bench.apply_tuning(Engine(), "no_such_shape=3")


def test_every_named_profile_exists_and_is_text():
    # the ncu summaries that bench.py, the documents and the summaries themselves cite
    import glob
    import re
    prof = os.path.join(ROOT, "profiles")
    sources = [os.path.join(ROOT, f) for f in ("bench.py", "DESIGN.md", "README.md", "INTEGRATION.md")]
    sources += glob.glob(os.path.join(ROOT, "pandemicthrust_gb300", "*.py")) + glob.glob(os.path.join(prof, "*"))
    named = set()
    for path in sources:
        if not os.path.isfile(path):
            continue
        text = open(path, encoding="utf-8").read()
        named.update(re.findall(r"profiles/([A-Za-z0-9_.-]+\.(?:md|txt))", text))
        if os.path.dirname(path) == prof:
            named.update(re.findall(r"`((?:ncu|launches)_[A-Za-z0-9_.-]+\.md)`", text))
    assert named
    for name in sorted(named):
        assert os.path.isfile(os.path.join(prof, name)), name
    for path in glob.glob(os.path.join(prof, "*")):
        assert path.endswith((".md", ".txt")), path
