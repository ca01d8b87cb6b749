"""The oracle at the headline size (50M persons) against the reference's own kernels:
setup tables and the first days' bins, infected counts and counter offsets from
tests/golden/headline_50M_100d.json.  The whole 100 days run on the GPU
(test_gpu_headline.py) and in the benchmark, where the oracle's first days are also
compared with the GPU's."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle.oracle import Oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "headline_50M_100d.json")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.skipif(not os.path.exists(GOLDEN), reason="headline golden fixture not generated")
def test_oracle_setup_and_first_days_at_50M_match_reference_kernels(oracle_built):
    with open(GOLDEN) as fh:
        g = json.load(fh)
    o = Oracle(g["params"], g["seed"], threads=os.cpu_count() or 1)
    o.setup()
    v = o.view()
    s = g["setup"]
    assert (v["N"], v["H"], v["L"], v["adults"], v["rand_offset"]) == (s["N"], s["H"], s["L"], s["adults"],
                                                                       s["rand_offset"])
    for k in ("age", "household", "workplace", "workplace_people", "workplace_offset"):
        assert digest(v[k]) == s[k], k
    for d in range(2):
        rc, c, i = o.step_day()
        ref = g["days"][d]
        assert (rc, c, i, o.view()["rand_offset"]) == (ref["rc"], ref["counts"], ref["infected"],
                                                       ref["rand_offset"]), d
    o.close()
