"""The intervention extensions on the CPU oracle (no reference counterpart): neutral
values change nothing, and each intervention lowers transmission.  Argument checks of
the C ABI need no device."""
import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import Oracle, make_params

BASE = make_params(max_days=40, r_pandemic=1.9, r_seasonal=1.7, initial_pandemic=20, initial_seasonal=20,
                   people_scaling=0.02, location_scaling=0.02)


def run_oracle(iv=None, seed=314):
    o = Oracle(BASE, seed)
    if iv is not None:
        o.set_interventions(**iv)
    o.setup()
    rows = []
    while True:
        rc, counts, infected = o.step_day()
        if rc == 2:  # max_days already run: no row
            break
        rows.append(counts)
        if rc != 0:
            break
    v = o.view()
    o.close()
    return np.array(rows), v


def attack(v):
    # infections over the run, both strains: persons with a generation (vaccinated
    # persons start recovered but were never infected)
    return int(np.sum(v["gen_p"] != 255) + np.sum(v["gen_s"] != 255))


def test_neutral_interventions_are_the_reference(oracle_built):
    rows0, v0 = run_oracle(None)
    rows1, v1 = run_oracle(dict(school_closure_start=0, school_closure_days=0, workplace_absenteeism=0.0,
                                vaccination_coverage=0.0))
    assert np.array_equal(rows0, rows1)
    for k in ("status_p", "status_s", "gen_p", "gen_s"):
        assert np.array_equal(v0[k], v1[k])


@pytest.mark.parametrize("iv", [
    dict(vaccination_coverage=0.5),
    dict(school_closure_start=0, school_closure_days=40),
    dict(workplace_absenteeism=0.6),
])
def test_each_intervention_lowers_the_attack(oracle_built, iv):
    _, base = run_oracle(None)
    rows, v = run_oracle(iv)
    assert attack(v) < attack(base)
    if "vaccination_coverage" in iv:
        vacc = (v["status_p"] == 0) & (v["gen_p"] == 255) & (v["status_s"] == 0) & (v["gen_s"] == 255)
        frac = vacc.mean()
        assert 0.45 < frac < 0.55  # about half the population starts immune


@pytest.mark.parametrize("bad", [
    dict(vaccination_coverage=1.5), dict(workplace_absenteeism=-0.1), dict(school_closure_days=-1),
    dict(school_closure_start=-3, school_closure_days=2),
])
def test_invalid_interventions_are_rejected(native_lib, bad):
    sim = pt.PandemicSim(BASE, 1)
    with pytest.raises(pt.PtError) as e:
        sim.set_interventions(bad)
    assert e.value.code == -1
    sim.close()
    b = pt.PandemicBatch([BASE, BASE], [1, 2])
    with pytest.raises(pt.PtError) as e:
        b.set_interventions([{}, bad])
    assert e.value.code == -1 and "instance 1" in str(e.value)
    b.close()
