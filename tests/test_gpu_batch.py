"""Batches of simulations against the same simulations run alone, bit for bit.

Instance k of a batch must reproduce pt_create(params[k], seeds[k]) run by itself:
every statistics row, the generation counts, every person's final state and the
setup tables.  The single-simulation path is checked against the oracle elsewhere,
so these comparisons carry the oracle's pin over to every instance of a batch."""
import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import Oracle, make_params

pytestmark = pytest.mark.gpu

# Uneven sizes, parameters and stopping days: the C1 shape, a larger population, a
# tiny one below one person tile, an epidemic that dies out, one with no seeds (stops
# on day 0), a shorter max_days, and a symptomatic/asymptomatic mix with more
# locations than persons imply.
MIXED = [
    (make_params(max_days=30, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10, initial_seasonal=10,
                 people_scaling=0.04248, location_scaling=0.04248), 12345),
    (make_params(max_days=40, r_pandemic=1.8, r_seasonal=1.3, initial_pandemic=30, initial_seasonal=30,
                 people_scaling=0.2, location_scaling=0.2), 7),
    (make_params(max_days=30, r_pandemic=2.0, r_seasonal=1.6, initial_pandemic=3, initial_seasonal=2,
                 people_scaling=0.001, location_scaling=0.001), 99),
    (make_params(max_days=60, r_pandemic=0.4, r_seasonal=0.3, initial_pandemic=2, initial_seasonal=1,
                 people_scaling=0.01, location_scaling=0.01), 5),
    (make_params(max_days=30, r_pandemic=1.5, r_seasonal=1.5, initial_pandemic=0, initial_seasonal=0,
                 people_scaling=0.01, location_scaling=0.01), 11),
    (make_params(max_days=5, r_pandemic=1.7, r_seasonal=1.2, initial_pandemic=20, initial_seasonal=20,
                 people_scaling=0.05, location_scaling=0.05), 2024),
    (make_params(max_days=35, r_pandemic=1.6, r_seasonal=1.4, initial_pandemic=15, initial_seasonal=25,
                 people_scaling=0.03, location_scaling=0.09, percent_symptomatic=0.6, asymp_factor=0.4), -17),
]


def standalone(params, seed):
    sim = pt.PandemicSim(params, seed)
    sim.setupSim()
    counts, infected = sim.runToCompletion()
    gp, gs = sim.final_gen_counts()
    out = dict(counts=counts, infected=infected, gen_p=gp, gen_s=gs, state=sim.person_state(),
               population=sim.population(), info=sim.info())
    sim.close()
    return out


def assert_instance_equal(b, k, ref, gen_p, gen_s):
    counts, infected = b.counts(k)
    assert np.array_equal(counts, ref["counts"]), k
    assert np.array_equal(infected, ref["infected"]), k
    assert np.array_equal(gen_p[k], ref["gen_p"]) and np.array_equal(gen_s[k], ref["gen_s"]), k
    st = b.person_state(k)
    for key, v in ref["state"].items():
        assert np.array_equal(st[key], v), (k, key, np.nonzero(st[key] != v)[0][:8])
    info = b.info(k)
    for key in ("number_people", "number_households", "number_workplaces", "number_adults", "days_run",
                "current_day", "infected_count", "rand_offset", "max_day_of_peak", "max_infected_proportion"):
        assert info[key] == ref["info"][key], (k, key)


def test_mixed_batch_equals_standalone_runs(native_lib):
    refs = [standalone(p, s) for p, s in MIXED]
    b = pt.PandemicBatch([p for p, _ in MIXED], [s for _, s in MIXED])
    b.setup()
    k, persons, padded = b.size()
    assert k == len(MIXED) and persons == sum(r["info"]["number_people"] for r in refs)
    assert padded % 4096 == 0 and padded >= persons
    for i, ref in enumerate(refs):
        pop = b.population(i)
        for key, v in ref["population"].items():
            assert np.array_equal(pop[key], v), (i, key)
    b.run()
    gp, gs = b.final_gen_counts()
    for i, ref in enumerate(refs):
        assert_instance_equal(b, i, ref, gp, gs)
    # the instance with no seeds stops on day 0; the short one at its max_days
    assert list(b.days_run()) == [len(r["infected"]) for r in refs]
    assert b.days_run()[4] == 1 and b.days_run()[5] == 5
    b.close()


# Above about 19.9M persons (four tiles per block, eight blocks per SM on 152 SMs) the
# sweep's count blocks take four person tiles each and its emit a warp per tile; with
# uneven instances, some count blocks span two instances and add up two bin rows.
LARGE = [
    (make_params(max_days=20, r_pandemic=1.8, r_seasonal=1.3, initial_pandemic=60, initial_seasonal=40,
                 people_scaling=ps, location_scaling=10 * ps), seed)
    for ps, seed in ((2.4, 31), (1.7, 32), (2.6, 33), (1.3, 34), (2.1, 35))
]


def test_large_batch_with_multi_tile_sweep_blocks_equals_standalone_runs(native_lib):
    torch = pytest.importorskip("torch")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    b = pt.PandemicBatch([p for p, _ in LARGE], [s for _, s in LARGE])
    b.setup()
    k, persons, padded = b.size()
    if padded // 4096 < 4 * 8 * sms:
        b.close()
        pytest.skip("batch below the multi-tile sweep size on this GPU")
    b.run()
    gp, gs = b.final_gen_counts()
    for i, (p, s) in enumerate(LARGE):
        ref = standalone(p, s)
        assert_instance_equal(b, i, ref, gp, gs)
    b.close()


def test_step_day_equals_run_and_reset_repeats(native_lib):
    params = [p for p, _ in MIXED[:4]]
    seeds = [s for _, s in MIXED[:4]]
    b = pt.PandemicBatch(params, seeds)
    b.setup()
    b.run()
    first = [b.counts(k) for k in range(4)]
    gp1, gs1 = b.final_gen_counts()
    b.reset_epidemic()
    b.run()  # replays the captured day loop
    gp2, gs2 = b.final_gen_counts()
    for k in range(4):
        c, i = b.counts(k)
        assert np.array_equal(c, first[k][0]) and np.array_equal(i, first[k][1])
    assert np.array_equal(gp1, gp2) and np.array_equal(gs1, gs2)
    b.reset_epidemic()
    days = 0
    while True:
        rc, running = b.step_day()
        days += 1
        if rc != pt.PT_OK or running == 0:
            break
    assert days <= max(p["max_days"] for p in params)
    for k in range(4):
        c, i = b.counts(k)
        assert np.array_equal(c, first[k][0]) and np.array_equal(i, first[k][1]), k
    b.close()


def test_replicates_and_scenarios_like_the_batched_workload(native_lib):
    # a small version of the batched workload: uneven sizes (log-uniform), R per
    # strain uniform in [1.1, 2.0], seed = 1000 + instance, 10 + 10 seed infections
    rng = np.random.default_rng(20240)
    params, seeds = [], []
    for k in range(12):
        n = float(np.exp(rng.uniform(np.log(2e4), np.log(3e5))))
        p = n / 2.354e6
        params.append(make_params(max_days=45, r_pandemic=float(rng.uniform(1.1, 2.0)),
                                  r_seasonal=float(rng.uniform(1.1, 2.0)), initial_pandemic=10,
                                  initial_seasonal=10, people_scaling=p, location_scaling=p))
        seeds.append(1000 + k)
    b = pt.PandemicBatch(params, seeds)
    b.setup()
    before = pt.launch_count()
    b.run()
    batch_launches = pt.launch_count() - before
    gp, gs = b.final_gen_counts()
    for k in range(12):
        ref = standalone(params[k], seeds[k])
        assert_instance_equal(b, k, ref, gp, gs)
    b.close()
    # the day loop launches the same kernels whatever the number of instances; only
    # the radix passes (one per 8 bits of the total bucket count) can differ
    one = pt.PandemicBatch(params[:1], seeds[:1])
    one.setup()
    before = pt.launch_count()
    one.run()
    one_launches = pt.launch_count() - before
    assert one_launches <= batch_launches <= one_launches + 2 * 45
    one.close()


def test_batch_instance_matches_oracle_directly(native_lib, oracle_built):
    p, seed = MIXED[0]
    b = pt.PandemicBatch([MIXED[2][0], p, MIXED[3][0]], [MIXED[2][1], seed, MIXED[3][1]])
    b.setup()
    b.run()
    counts, infected = b.counts(1)
    o = Oracle(p, seed)
    o.setup()
    for day in range(len(infected)):
        r = o.step_day()
        assert np.array_equal(counts[day], np.asarray(r[1])) and infected[day] == r[2], day
    v = o.view()
    st = b.person_state(1)
    for key in ("status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s"):
        assert np.array_equal(st[key], v[key]), key
    o.close()
    b.close()
