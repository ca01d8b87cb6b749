"""Host logic of the native library that needs no GPU: exports, constants.csv and
seed.txt parsing, parameter validation, seeds and scaling."""
import ctypes
import os
import re

import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import Oracle, constants_csv_text, make_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "pandemic_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(pt_\w+)\s*\(", txt, flags=re.M)))


def test_library_exports_every_declared_symbol(native_lib):
    syms = declared_symbols()
    assert len(syms) >= 17
    for name in syms:
        assert hasattr(native_lib, name), name
    assert set(syms) <= set(pt.EXPORTS) | set(syms)


def test_params_from_reference_constants_csv(native_lib, tmp_path):
    # the reference's own default file layout (PandemicThrust/PandemicThrust/constants.csv)
    f = tmp_path / "constants.csv"
    f.write_text("constants,max_days,reproduction_number_pandemic,reproduction_number_seasonal,"
                 "initial_infected_pandemic,initial_infected_seasonal,people_scaling_factor,"
                 "location_scaling_factor,percent_symptomatic,asymp_factor\n"
                 "constants,100,1.8,1.3,30,30,1,1,1,0\n")
    p = pt.Params()
    assert native_lib.pt_params_from_csv(str(f).encode(), ctypes.byref(p)) == 0
    assert (p.max_days, p.initial_pandemic, p.initial_seasonal) == (100, 30, 30)
    assert p.r_pandemic == np.float32(1.8) and p.r_seasonal == np.float32(1.3)
    assert (p.people_scaling, p.location_scaling, p.percent_symptomatic, p.asymp_factor) == (1, 1, 1, 0)


def test_params_roundtrip_and_errors(native_lib, tmp_path):
    d = make_params(max_days=30, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10, initial_seasonal=10,
                    people_scaling=0.04248, location_scaling=0.04248)
    f = tmp_path / "constants.csv"
    f.write_text(constants_csv_text(d))
    p = pt.Params()
    assert native_lib.pt_params_from_csv(str(f).encode(), ctypes.byref(p)) == 0
    assert p.people_scaling == np.float32(0.04248)
    assert native_lib.pt_params_from_csv(str(tmp_path / "missing.csv").encode(), ctypes.byref(p)) == -2
    bad = tmp_path / "bad.csv"
    bad.write_text("header only\n")
    assert native_lib.pt_params_from_csv(str(bad).encode(), ctypes.byref(p)) == -3
    seed = tmp_path / "seed.txt"
    seed.write_text("12345\n")
    v = ctypes.c_int(0)
    assert native_lib.pt_seed_from_file(str(seed).encode(), ctypes.byref(v)) == 0 and v.value == 12345
    assert native_lib.pt_seed_from_file(str(tmp_path / "nope").encode(), ctypes.byref(v)) == -2


@pytest.mark.parametrize("field,value", [("max_days", 256), ("max_days", -1), ("initial_pandemic", -3),
                                         ("people_scaling", 0.0), ("location_scaling", -1.0)])
def test_invalid_parameters_rejected(native_lib, field, value):
    d = make_params()
    d[field] = value
    with pytest.raises(pt.PtError) as e:
        pt.PandemicSim(d, 1)
    assert e.value.code == -1


@pytest.mark.parametrize("params,seed", [
    (make_params(people_scaling=0.04248, location_scaling=0.04248), 12345),
    (make_params(people_scaling=21.24044, location_scaling=212.4, r_pandemic=1.5, r_seasonal=1.2), 777),
    (make_params(percent_symptomatic=0.6, asymp_factor=0.3), -5),
])
def test_create_derives_seeds_and_scaling_like_oracle(native_lib, oracle_built, params, seed):
    sim = pt.PandemicSim(params, seed)  # no device work until setupSim
    info = sim.info()
    o = Oracle(params, seed)
    v = o.view()
    assert info["seeds"] == v["seeds"]
    assert info["number_households"] == v["H"] and info["number_workplaces"] == v["L"]
    assert info["type_count"] == v["type_count"] and info["type_offset"] == v["type_offset"]
    assert np.array(info["infectiousness"], np.float32).tobytes() == v["infectiousness"].tobytes()
    sim.close()
    o.close()


def test_config2_scaling_matches_plan(native_lib):
    # 50M-person workload: 21.24M households, 2,718,720 locations (lscale = 10 x pscale)
    sim = pt.PandemicSim(make_params(people_scaling=21.24044, location_scaling=212.4044), 777)
    info = sim.info()
    assert info["number_households"] == 21240440
    assert 2_700_000 < info["number_workplaces"] < 2_750_000
    sim.close()
