"""Launch shapes and the tuner: every shape gives bit-identical results.

The day's kernels take their launch shapes at run time (pt_tuning): the infection
kernel as one thread per infector or eight lanes per infector (warp-cooperative
contacts), its grid, and the radix passes' persistent grid.  The reference fixes its
grids at compile time (device_K20.h:4-8).  Results must not depend on the shape: each
candidate is run against the default and against the oracle, weekdays and weekends,
with and without interventions, alone and in a batch."""
import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import Oracle, make_params

pytestmark = pytest.mark.gpu

SHAPES = [dict(infect_coop=0, infect_blocks_per_sm=8, radix_blocks_per_sm=3, sched_tf=0, dense_level=0,
               radix_threads=256),
          dict(infect_coop=1, infect_blocks_per_sm=6, radix_blocks_per_sm=2, sched_tf=1, dense_level=1,
               radix_threads=512),
          dict(infect_coop=1, infect_blocks_per_sm=1, radix_blocks_per_sm=1, sched_tf=2, dense_level=2,
               radix_threads=512),
          dict(infect_coop=0, infect_blocks_per_sm=1, radix_blocks_per_sm=1, sched_tf=2, dense_level=3,
               radix_threads=256),
          dict(infect_coop=1, infect_blocks_per_sm=32, radix_blocks_per_sm=4, sched_tf=1, dense_level=1,
               radix_threads=256)]

FIELDS = ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s")


def run_sim(p, seed, shape, iv=None):
    sim = pt.PandemicSim(p, seed)
    sim.set_tuning(shape)
    if iv:
        sim.set_interventions(iv)
    sim.setupSim()
    assert sim.tuning() == shape
    c, i = sim.runToCompletion()
    st = sim.person_state()
    g = sim.final_gen_counts()
    sim.close()
    return c, i, st, g


@pytest.mark.parametrize("iv", [None, dict(school_closure_start=3, school_closure_days=12,
                                           workplace_absenteeism=0.2, vaccination_coverage=0.1)])
def test_every_shape_matches_the_oracle(native_lib, oracle_built, iv):
    p = make_params(max_days=24, people_scaling=0.03, location_scaling=0.03, r_pandemic=2.2, r_seasonal=1.8,
                    percent_symptomatic=0.8, asymp_factor=0.3)
    o = Oracle(p, 9)
    if iv:
        o.set_interventions(**iv)
    o.setup()
    rows = []
    while True:
        rc, c, i = o.step_day()
        if rc == 2:
            break
        rows.append((c, i))
        if rc == 1:
            break
    v = o.view()
    og = o.gen_counts()
    o.close()
    for shape in SHAPES:
        c, i, st, g = run_sim(p, 9, shape, iv)
        assert len(i) == len(rows), shape
        for d, (oc, oi) in enumerate(rows):
            assert c[d].tolist() == oc and i[d] == oi, (shape, d)
        for k in FIELDS:
            assert np.array_equal(st[k], v[k]), (shape, k)
        assert np.array_equal(g[0], og[0]) and np.array_equal(g[1], og[1]), shape


def test_batch_shapes_and_autotune_are_identical(native_lib):
    params = [make_params(max_days=30, people_scaling=s, location_scaling=s, r_pandemic=r, r_seasonal=1.5)
              for s, r in ((0.004, 2.4), (0.02, 1.9), (0.05, 2.1), (0.012, 1.4))]
    seeds = [11, 12, 13, 14]
    ref = None
    for shape in SHAPES + ["auto"]:
        b = pt.PandemicBatch(params, seeds)
        b.setup()
        if shape == "auto":
            chosen = b.autotune(days=12)
            assert chosen["infect_coop"] in (0, 1) and 1 <= chosen["radix_blocks_per_sm"] <= 4
            assert b.tuning() == chosen
        else:
            b.set_tuning(shape)
        b.run()
        out = [b.counts(k) for k in range(4)], b.final_gen_counts(), [b.person_state(k) for k in range(4)]
        b.close()
        if ref is None:
            ref = out
            continue
        for k in range(4):
            assert np.array_equal(out[0][k][0], ref[0][k][0]) and np.array_equal(out[0][k][1], ref[0][k][1])
            for f in FIELDS:
                assert np.array_equal(out[2][k][f], ref[2][k][f]), (shape, k, f)
        assert np.array_equal(out[1][0], ref[1][0]) and np.array_equal(out[1][1], ref[1][1])


def test_autotune_on_a_plain_simulation_then_run_equals_default(native_lib):
    p = make_params(max_days=20, people_scaling=0.05, location_scaling=0.05, r_pandemic=2.0)
    c0, i0, s0, g0 = run_sim(p, 21, SHAPES[0])
    sim = pt.PandemicSim(p, 21)
    sim.setupSim()
    t = sim.autotune()
    assert sim.tuning() == t
    c, i = sim.runToCompletion()
    st = sim.person_state()
    sim.close()
    assert np.array_equal(c, c0) and np.array_equal(i, i0)
    for k in FIELDS:
        assert np.array_equal(st[k], s0[k]), k


def test_bad_shapes_are_rejected(native_lib):
    sim = pt.PandemicSim(make_params(max_days=2, people_scaling=0.001, location_scaling=0.001), 1)
    ok = dict(infect_coop=0, infect_blocks_per_sm=4, radix_blocks_per_sm=1, sched_tf=0, dense_level=0,
              radix_threads=256)
    for bad in (dict(ok, infect_coop=2), dict(ok, infect_blocks_per_sm=0), dict(ok, radix_blocks_per_sm=5),
                dict(ok, sched_tf=3), dict(ok, dense_level=4), dict(ok, radix_threads=384),
                dict(ok, radix_threads=512, radix_blocks_per_sm=3)):
        with pytest.raises(pt.PtError):
            sim.set_tuning(bad)
    sim.close()
