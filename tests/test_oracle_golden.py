"""The CPU oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py): Random123 blocks, the C library's rand() sequence,
host_functions.cpp regeneration and whole runs of the reference's kernels."""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

from oracle.oracle import Oracle, glibc_rand, oracle_lib, threefry2x32, threefry2x64

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name)) as fh:
        return json.load(fh)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_threefry2x64_matches_random123(oracle_built):
    g = load("rng.json")
    for c, k0, k1, o0, o1 in g["threefry2x64"]:
        assert threefry2x64([int(c), int(c)], [int(k0), int(k1)]) == [int(o0), int(o1)]


def test_threefry2x32_matches_random123(oracle_built):
    g = load("rng.json")
    for c0, c1, k0, k1, o0, o1 in g["threefry2x32"]:
        assert threefry2x32([c0, c1], [k0, k1]) == [o0, o1]


def test_glibc_rand_matches_libc(oracle_built):
    g = load("rng.json")
    for seed, seq in g["libc_rand"].items():
        assert glibc_rand(int(seed), len(seq)) == seq


PARAMS = {
    "c1": dict(max_days=30, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10, initial_seasonal=10,
               people_scaling=0.04248, location_scaling=0.04248, percent_symptomatic=1.0, asymp_factor=0.0),
    "lscale10": dict(max_days=40, r_pandemic=2.0, r_seasonal=1.5, initial_pandemic=5, initial_seasonal=3,
                     people_scaling=0.01, location_scaling=0.1, percent_symptomatic=1.0, asymp_factor=0.0),
    "c2_shape": dict(max_days=100, r_pandemic=1.8, r_seasonal=1.3, initial_pandemic=30, initial_seasonal=30,
                     people_scaling=0.42481, location_scaling=4.2481, percent_symptomatic=1.0, asymp_factor=0.0),
}
SEEDS = {"c1": 12345, "lscale10": 4242, "c2_shape": 777}


@pytest.mark.parametrize("name", ["c1", "lscale10", "c2_shape"])
def test_regeneration_matches_host_functions(oracle_built, name):
    g = load("regen.json")[name]
    o = Oracle(PARAMS[name], SEEDS[name])
    o.setup()
    v = o.view()
    for k in ("N", "H", "L", "seeds", "type_count", "type_offset", "workplace_rand_offset"):
        assert v[k] == g[k], k
    assert v["infectiousness"].tolist() == pytest.approx(g["infectiousness"], rel=0, abs=0)
    lib = oracle_lib()
    for idx, age, wp in g["workplace"]:
        assert lib.ptor_recalc_workplace(o.h, idx, age) == wp
    for off, idx, age, prof, d1, d2 in g["weekday"]:
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        assert lib.ptor_recalc_weekday_errands(o.h, off, idx, age, ctypes.byref(a), ctypes.byref(b)) == prof
        assert (a.value, b.value) == (d1, d2)
    for off, idx, dests in g["weekend"]:
        out = (ctypes.c_int * 3)()
        lib.ptor_recalc_weekend_errands(o.h, off, idx, out)
        assert list(out) == dests
    o.close()


@pytest.mark.parametrize("name", ["c1_100k_30d", "default_p0.1_asymp", "small_lscale10"])
def test_whole_run_matches_reference_kernels(oracle_built, name):
    g = load("runs.json")[name]
    o = Oracle(g["params"], g["seed"])
    o.setup()
    v = o.view()
    s = g["setup"]
    for k in ("N", "H", "L", "adults", "children", "rand_offset"):
        assert v[k] == s[k], k
    for k in ("age", "household", "household_offset", "workplace", "workplace_people", "workplace_offset",
              "status_p", "status_s"):
        assert digest(v[k]) == s[k], k
    for day, ref in enumerate(g["days"]):
        rc, counts, infected = o.step_day()
        assert (rc, counts, infected) == (ref["rc"], ref["counts"], ref["infected"]), day
        v = o.view()
        assert v["rand_offset"] == ref["rand_offset"], day
        for k in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s"):
            assert digest(v[k]) == ref[k], (day, k)
        assert digest(v["infected"][:infected]) == ref["infected_list"], day
        if ref["errand_people"] is not None:
            assert digest(v["errand_people"]) == ref["errand_people"], day
            assert digest(v["errand_offset"]) == ref["errand_offset"], day
    gp, gs = o.gen_counts()
    assert gp.tolist() == g["gen_p"]
    assert gs.tolist() == g["gen_s"]
    o.close()
