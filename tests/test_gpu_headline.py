"""The headline workload, 50M persons x 100 days, bit for bit against the reference.

tests/golden/headline_50M_100d.json is a run of the reference's own kernels compiled
for the host (one thread: the canonical order; tests/golden/make_golden.py
--headline): the setup tables' digests, every day's 16 status bins, infected count and
counter offset, the final per-person state's digests and the generation counts.  The
CUDA path runs the same workload through pt_run (the day loop as one CUDA graph) and
must match all of it exactly."""
import hashlib
import json
import os

import numpy as np
import pytest

import pandemicthrust_gb300 as pt

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "headline_50M_100d.json")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.skipif(not os.path.exists(GOLDEN), reason="headline golden fixture not generated")
def test_headline_50M_100_days_matches_reference_kernels(native_lib):
    with open(GOLDEN) as fh:
        g = json.load(fh)
    sim = pt.PandemicSim(g["params"], g["seed"])
    sim.setupSim()
    info = sim.info()
    s = g["setup"]
    assert (info["number_people"], info["number_households"], info["number_workplaces"]) == (s["N"], s["H"], s["L"])
    assert info["number_adults"] == s["adults"] and info["rand_offset"] == s["rand_offset"]
    pop = sim.population()
    for k in ("household", "workplace", "workplace_people", "workplace_offset"):
        assert digest(pop[k]) == s[k], k
    del pop
    assert digest(sim.person_state()["age"]) == s["age"]
    counts, infected = sim.runToCompletion()
    assert len(infected) == len(g["days"])
    for d, ref in enumerate(g["days"]):
        assert counts[d].tolist() == ref["counts"] and int(infected[d]) == ref["infected"], d
    assert sim.info()["rand_offset"] == g["days"][-1]["rand_offset"]
    st = sim.person_state()
    for k, v in g["final"].items():
        assert digest(st[k]) == v, k
    gp, gs = sim.final_gen_counts()
    assert gp.tolist() == g["gen_p"] and gs.tolist() == g["gen_s"]
    sim.close()
