"""CUDA path against the CPU oracle and the reference-derived golden runs, bit for bit.

Every comparison is exact: the path is integer/byte work plus float lookups that the
reference performs in IEEE single precision, reproduced with round-to-nearest
intrinsics, so the tolerance is zero."""
import hashlib
import json
import os

import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import Oracle, make_params

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

C1 = make_params(max_days=30, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10, initial_seasonal=10,
                 people_scaling=0.04248, location_scaling=0.04248)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def gpu_state(sim):
    return sim.person_state()


def assert_setup_equal(sim, o):
    info = sim.info()
    v = o.view()
    assert info["number_people"] == v["N"]
    assert info["number_households"] == v["H"]
    assert info["number_workplaces"] == v["L"]
    assert info["number_adults"] == v["adults"]
    assert info["rand_offset"] == v["rand_offset"]
    pop = sim.population()
    for k in ("household", "household_offset", "workplace", "workplace_people", "workplace_offset"):
        assert np.array_equal(pop[k], v[k]), k
    st = gpu_state(sim)
    for k in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s", "age"):
        assert np.array_equal(st[k], v[k]), k


def assert_day_equal(sim, o, day, check_tables=True):
    g = sim.step_day()
    r = o.step_day()
    assert g[0] == r[0] and g[1] == r[1] and g[2] == r[2], (day, g, r)
    v = o.view()
    st = gpu_state(sim)
    for k in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s"):
        assert np.array_equal(st[k], v[k]), (day, k, np.nonzero(st[k] != v[k])[0][:8])
    if r[0] == 0:
        assert sim.info()["rand_offset"] == v["rand_offset"], day
        if check_tables:
            t = sim.day_tables()
            assert np.array_equal(t["infected"][:r[2]], v["infected"]), day
            assert t["entries"] == v["errand_entries"] and t["buckets"] == v["errand_buckets"]
            assert np.array_equal(t["keys"], v["errand_keys"]), day
            assert np.array_equal(t["offsets"], v["errand_offset"]), day
            assert np.array_equal(t["people"], v["errand_people"]), day
    return r[0]


def test_setup_matches_oracle(native_lib, oracle_built):
    sim = pt.PandemicSim(C1, 12345)
    sim.setupSim()
    o = Oracle(C1, 12345)
    o.setup()
    assert_setup_equal(sim, o)
    sim.close()
    o.close()


def test_config1_days_match_oracle_stage_by_stage(native_lib, oracle_built):
    sim = pt.PandemicSim(C1, 12345)
    sim.set_full_tables(True)
    sim.setupSim()
    o = Oracle(C1, 12345)
    o.setup()
    for day in range(C1["max_days"]):
        if assert_day_equal(sim, o, day) != 0:
            break
    gp, gs = sim.final_gen_counts()
    op, os_ = o.gen_counts()
    assert np.array_equal(gp, op) and np.array_equal(gs, os_)
    sim.close()
    o.close()


@pytest.mark.parametrize("name", ["c1_100k_30d", "default_p0.1_asymp", "small_lscale10"])
def test_whole_run_matches_reference_golden(native_lib, name):
    with open(os.path.join(GOLDEN, "runs.json")) as fh:
        g = json.load(fh)[name]
    sim = pt.PandemicSim(g["params"], g["seed"])
    sim.setupSim()
    pop = sim.population()
    assert digest(pop["workplace_people"]) == g["setup"]["workplace_people"]
    assert digest(pop["household_offset"]) == g["setup"]["household_offset"]
    for day, ref in enumerate(g["days"]):
        rc, counts, infected = sim.step_day()
        assert (rc, counts, infected) == (ref["rc"], ref["counts"], ref["infected"]), day
        st = sim.person_state()
        for k in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s"):
            assert digest(st[k]) == ref[k], (day, k)
    gp, gs = sim.final_gen_counts()
    assert gp.tolist() == g["gen_p"] and gs.tolist() == g["gen_s"]
    sim.close()


def test_run_on_device_equals_day_steps(native_lib):
    p = make_params(max_days=40, people_scaling=0.05, location_scaling=0.05, percent_symptomatic=0.7,
                    asymp_factor=0.4)
    a = pt.PandemicSim(p, 99)
    a.setupSim()
    counts, infected = a.runToCompletion()
    st_a = a.person_state()
    b = pt.PandemicSim(p, 99)
    b.setupSim()
    rows = []
    while True:
        rc, c, i = b.step_day()
        if rc == pt.PT_FINISHED:
            break
        rows.append((c, i))
        if rc == pt.PT_DONE:
            break
    assert len(rows) == len(counts)
    for d, (c, i) in enumerate(rows):
        assert counts[d].tolist() == c and infected[d] == i
    st_b = b.person_state()
    for k in st_a:
        assert np.array_equal(st_a[k], st_b[k]), k
    assert a.info()["max_infected_proportion"] == b.info()["max_infected_proportion"]
    a.close()
    b.close()


def test_lazy_buckets_equal_full_tables(native_lib):
    # materialising only the buckets infected persons visit must not change anything
    p = make_params(max_days=60, people_scaling=0.1, location_scaling=0.1, percent_symptomatic=0.8,
                    asymp_factor=0.2)
    runs = []
    for full in (False, True):
        sim = pt.PandemicSim(p, 31)
        sim.set_full_tables(full)
        sim.setupSim()
        counts, infected = sim.runToCompletion()
        info = sim.info()
        runs.append((counts, infected, sim.person_state(), info))
        sim.close()
    (c0, i0, s0, f0), (c1, i1, s1, f1) = runs
    assert np.array_equal(c0, c1) and np.array_equal(i0, i1)
    for k in s0:
        assert np.array_equal(s0[k], s1[k]), k
    assert f1["bucket_entries_materialised"] == f1["bucket_entries_scheduled"]
    assert f0["bucket_entries_materialised"] < f0["bucket_entries_scheduled"]


def test_deterministic_and_resettable(native_lib):
    p = make_params(max_days=25, people_scaling=0.08, location_scaling=0.02)
    sim = pt.PandemicSim(p, 5)
    sim.setupSim()
    c1, i1 = sim.runToCompletion()
    s1 = sim.person_state()
    sim.reset_epidemic()
    c2, i2 = sim.runToCompletion()
    s2 = sim.person_state()
    assert np.array_equal(c1, c2) and np.array_equal(i1, i2)
    for k in s1:
        assert np.array_equal(s1[k], s2[k]), k
    sim.close()


def test_config2_shape_one_million_matches_oracle(native_lib, oracle_built):
    # 1M persons with the 50M workload's location ratio (lscale = 10 x pscale)
    p = make_params(max_days=21, r_pandemic=1.5, r_seasonal=1.2, initial_pandemic=100, initial_seasonal=100,
                    people_scaling=0.42481, location_scaling=4.2481)
    sim = pt.PandemicSim(p, 777)
    sim.set_full_tables(True)
    sim.setupSim()
    o = Oracle(p, 777, threads=8)
    o.setup()
    assert_setup_equal(sim, o)
    for day in range(p["max_days"]):
        if assert_day_equal(sim, o, day, check_tables=(day % 7 in (0, 5))) != 0:
            break
    sim.close()
    o.close()


@pytest.mark.parametrize("params,seed", [
    (make_params(max_days=0, people_scaling=0.001, location_scaling=0.001), 3),
    (make_params(max_days=1, people_scaling=0.001, location_scaling=0.001), 3),
    (make_params(max_days=9, people_scaling=0.001, location_scaling=0.001, initial_pandemic=0,
                 initial_seasonal=0), 3),
    (make_params(max_days=60, people_scaling=0.00002, location_scaling=0.00001, initial_pandemic=2,
                 initial_seasonal=2, r_pandemic=4.0, r_seasonal=4.0), 11),
    (make_params(max_days=30, people_scaling=0.002, location_scaling=0.0001, r_pandemic=2.5), 8),
])
def test_edge_configurations_match_oracle(native_lib, oracle_built, params, seed):
    sim = pt.PandemicSim(params, seed)
    sim.setupSim()
    o = Oracle(params, seed)
    o.setup()
    assert_setup_equal(sim, o)
    for day in range(params["max_days"] + 1):
        g = sim.step_day()
        r = o.step_day()
        assert g == r, day
        if r[0] != 0:
            break
    st = sim.person_state()
    v = o.view()
    for k in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s"):
        assert np.array_equal(st[k], v[k]), k
    sim.close()
    o.close()


def test_launches_are_counted(native_lib):
    before = pt.launch_count()
    sim = pt.PandemicSim(make_params(max_days=3, people_scaling=0.01, location_scaling=0.01), 1)
    sim.setupSim()
    sim.runToCompletion()
    sim.close()
    assert pt.launch_count() > before
