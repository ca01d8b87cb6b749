"""Interventions on the GPU against the oracle's restatement, bit for bit, and in
batches against the same simulations run alone."""
import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import Oracle, make_params

pytestmark = pytest.mark.gpu

P = make_params(max_days=35, r_pandemic=1.8, r_seasonal=1.5, initial_pandemic=15, initial_seasonal=15,
                people_scaling=0.04248, location_scaling=0.04248)
IV = dict(school_closure_start=3, school_closure_days=17, workplace_absenteeism=0.25, vaccination_coverage=0.3)


def oracle_run(params, seed, iv):
    o = Oracle(params, seed)
    o.set_interventions(**iv)
    o.setup()
    rows = []
    while True:
        rc, counts, infected = o.step_day()
        if rc == 2:  # max_days already run: no row
            break
        rows.append((counts, infected))
        if rc != 0:
            break
    v = o.view()
    gp, gs = o.gen_counts()
    o.close()
    return rows, v, gp, gs


@pytest.mark.parametrize("iv", [IV, dict(vaccination_coverage=0.7), dict(school_closure_start=0,
                                                                         school_closure_days=35,
                                                                         workplace_absenteeism=0.5)])
def test_interventions_match_oracle(native_lib, oracle_built, iv):
    sim = pt.PandemicSim(P, 4242)
    sim.set_interventions(iv)
    sim.setupSim()
    counts, infected = sim.runToCompletion()
    rows, v, gp, gs = oracle_run(P, 4242, iv)
    assert len(rows) == len(infected)
    for d, (c, i) in enumerate(rows):
        assert list(counts[d]) == list(c) and infected[d] == i, d
    st = sim.person_state()
    for k in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s"):
        assert np.array_equal(st[k], v[k]), k
    g1, g2 = sim.final_gen_counts()
    assert np.array_equal(g1, gp) and np.array_equal(g2, gs)
    sim.close()


def test_interventions_after_setup_apply_at_reset(native_lib, oracle_built):
    sim = pt.PandemicSim(P, 99)
    sim.setupSim()
    sim.set_interventions(IV)
    sim.reset_epidemic()  # vaccination takes effect here
    counts, infected = sim.runToCompletion()
    rows, v, gp, gs = oracle_run(P, 99, IV)
    assert [int(x) for x in infected] == [r[1] for r in rows]
    sim.set_interventions({})
    sim.reset_epidemic()
    c0, i0 = sim.runToCompletion()
    rows0, _, _, _ = oracle_run(P, 99, {})
    assert [int(x) for x in i0] == [r[1] for r in rows0]
    sim.close()


def test_batch_with_mixed_interventions_equals_runs_alone(native_lib):
    params = [P, make_params(max_days=30, r_pandemic=1.6, r_seasonal=1.9, initial_pandemic=30, initial_seasonal=5,
                             people_scaling=0.02, location_scaling=0.03), P]
    seeds = [1, 2, 3]
    ivs = [IV, dict(workplace_absenteeism=0.3), {}]
    b = pt.PandemicBatch(params, seeds)
    b.set_interventions(ivs)
    b.setup()
    b.run()
    for k in range(3):
        sim = pt.PandemicSim(params[k], seeds[k])
        sim.set_interventions(ivs[k])
        sim.setupSim()
        c, i = sim.runToCompletion()
        bc, bi = b.counts(k)
        assert np.array_equal(c, bc) and np.array_equal(i, bi), k
        st, bst = sim.person_state(), b.person_state(k)
        for key in ("status_p", "status_s", "gen_p", "gen_s"):
            assert np.array_equal(st[key], bst[key]), (k, key)
        sim.close()
    b.close()
