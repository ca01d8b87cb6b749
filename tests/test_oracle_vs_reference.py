"""The oracle against the reference's kernels compiled for the host (oracle/_ref),
array by array and day by day.  Runs only where the reference tree was present when
oracle/build_ref.py ran; the committed golden fixtures cover the same ground elsewhere."""
import numpy as np
import pytest

from oracle import build_ref
from oracle.oracle import Oracle, RefSim, make_params, ref_available

if not ref_available():
    build_ref.build()

pytestmark = pytest.mark.skipif(not ref_available(), reason="reference-derived checker not built (no reference tree)")

ARRAYS = ["status_p", "status_s", "day_p", "day_s", "gen_p", "gen_s", "infected", "errand_keys",
          "errand_people", "errand_offset"]


@pytest.mark.parametrize("params,seed", [
    (make_params(max_days=21, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10, initial_seasonal=10,
                 people_scaling=0.04248, location_scaling=0.04248), 12345),
    (make_params(max_days=30, r_pandemic=3.0, r_seasonal=2.5, initial_pandemic=40, initial_seasonal=20,
                 people_scaling=0.02, location_scaling=0.005, percent_symptomatic=0.5, asymp_factor=0.5), -17),
    (make_params(max_days=12, people_scaling=0.003, location_scaling=0.02, initial_pandemic=3,
                 initial_seasonal=0), 1),
])
def test_oracle_tracks_reference_kernels(oracle_built, params, seed):
    o = Oracle(params, seed)
    r = RefSim(params, seed)
    o.setup()
    r.setup()
    vo, vr = o.view(), r.view()
    for k in ["N", "H", "L", "adults", "children", "rand_offset", "seeds", "type_count", "type_offset"]:
        assert vo[k] == vr[k], k
    for k in ["age", "household", "household_offset", "workplace", "workplace_people", "workplace_offset",
              "status_p", "status_s", "gen_p", "gen_s"]:
        assert np.array_equal(vo[k], vr[k]), k
    for day in range(params["max_days"] + 1):
        a, b = o.step_day(), r.step_day()
        assert a == b, day
        vo, vr = o.view(), r.view()
        assert vo["rand_offset"] == vr["rand_offset"], day
        for k in ARRAYS:
            assert np.array_equal(vo[k], vr[k]), (day, k)
        if a[0] != 0:
            break
    o.close()
    r.close()
