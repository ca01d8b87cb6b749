"""The output files the drop-in executables write (pt_output.cpp), checked on the CPU:
fed the oracle's per-day counts and generation counts, they must be byte-identical to
the files the oracle writes for the same run (output_infected_stats.csv,
output_rn.csv with its last-row and division-by-zero quirks, infected_max.txt)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import Oracle, make_params, oracle_run_to_files

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "pandemicthrust_gb300", "csrc")

SHIM = r'''
#include "pt_output.h"
extern "C" int shim_stats(const char *path, const int *counts, int rows)
{ return pto::write_infected_stats(path, counts, rows) ? 0 : 1; }
extern "C" int shim_rn(const char *path, const int *gp, const int *gs, int max_days, int persons)
{ return pto::write_rn(path, gp, gs, max_days, persons) ? 0 : 1; }
extern "C" int shim_max(const char *path, float proportion, int day)
{ return pto::write_infected_max(path, proportion, day) ? 0 : 1; }
extern "C" int shim_profile(const char *path, int days, const int *infected, const float *ms8)
{
    std::vector<pto::ProfileRow> rows;
    for (int d = 0; d < days; d++)
        pto::day_profile_rows(rows, d, (d % 7) >= 5, 1000, infected[d], ms8 + 8 * d);
    return pto::write_profile_log(path, rows) ? 0 : 1;
}
'''


@pytest.fixture(scope="module")
def writers(tmp_path_factory):
    d = tmp_path_factory.mktemp("shim")
    (d / "shim.cpp").write_text(SHIM)
    so = d / "libshim.so"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-shared", "-fPIC", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "include"), "-I", CSRC, os.path.join(CSRC, "pt_output.cpp"),
                           str(d / "shim.cpp"), "-o", str(so)])
    lib = ctypes.CDLL(str(so))
    ip = ctypes.POINTER(ctypes.c_int)
    lib.shim_stats.argtypes = [ctypes.c_char_p, ip, ctypes.c_int]
    lib.shim_rn.argtypes = [ctypes.c_char_p, ip, ip, ctypes.c_int, ctypes.c_int]
    lib.shim_max.argtypes = [ctypes.c_char_p, ctypes.c_float, ctypes.c_int]
    lib.shim_profile.argtypes = [ctypes.c_char_p, ctypes.c_int, ip, ctypes.POINTER(ctypes.c_float)]
    return lib


def _ints(a):
    a = np.ascontiguousarray(a, np.int32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


@pytest.mark.parametrize("params,seed", [
    (make_params(max_days=30, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10, initial_seasonal=10,
                 people_scaling=0.04248, location_scaling=0.04248), 12345),
    (make_params(max_days=40, r_pandemic=1.05, r_seasonal=0.9, initial_pandemic=3, initial_seasonal=2,
                 people_scaling=0.01, location_scaling=0.01), 7),
])
def test_writers_match_the_oracle_files(oracle_built, writers, tmp_path, params, seed):
    ref = tmp_path / "oracle"
    ref.mkdir()
    oracle_run_to_files(params, seed, str(ref))
    o = Oracle(params, seed)
    o.setup()
    rows, best, best_day = [], np.float32(0), 0
    while True:
        rc, counts, infected = o.step_day()
        if rc == 2:
            break
        day = len(rows)
        rows.append(counts)
        if rc == 1:
            break
        prop = np.float32(infected) / np.float32(o.view()["N"])
        if prop > best:
            best, best_day = prop, day
    gp, gs = o.gen_counts()
    N = o.view()["N"]
    o.close()
    mine = tmp_path / "mine"
    mine.mkdir()
    c, cp = _ints(np.array(rows).reshape(-1))
    assert writers.shim_stats(str(mine / "output_infected_stats.csv").encode(), cp, len(rows)) == 0
    g1, p1 = _ints(gp)
    g2, p2 = _ints(gs)
    assert writers.shim_rn(str(mine / "output_rn.csv").encode(), p1, p2, params["max_days"], N) == 0
    assert writers.shim_max(str(mine / "infected_max.txt").encode(), float(best), best_day) == 0
    for name in ("output_infected_stats.csv", "output_rn.csv", "infected_max.txt"):
        assert (mine / name).read_bytes() == (ref / name).read_bytes(), name


def test_profile_log_keeps_the_reference_profiler_format(writers, tmp_path):
    """profiler.cu:13 (header) and :72-76 (rows: "%d, %d, %s, %d, %f, %lf"); children
    are written before their parent; a day without infected ends after its first two
    rows, as the reference breaks out of the loop there."""
    import re
    days = 8
    infected = np.array([5, 9, 12, 20, 31, 40, 44, 0], np.int32)
    ms = np.arange(days * 8, dtype=np.float32).reshape(days, 8) / 8.0
    path = tmp_path / "profile_log.csv"
    ip = infected.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    assert writers.shim_profile(str(path).encode(), days, ip, ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
    lines = path.read_text().splitlines()
    assert lines[0] == ("day,stack_depth,function_name,problem_size,inclusive_time_milliseconds,"
                        "exclusive_time_milliseconds")
    rx = re.compile(r"^(\d+), (\d+), (\w+), (\d+), (\d+\.\d{6}), (\d+\.\d{6})$")
    rows = [rx.match(l).groups() for l in lines[1:]]
    by_day = {}
    for r in rows:
        by_day.setdefault(int(r[0]), []).append(r)
    weekday = [r[2] for r in by_day[0]]
    assert weekday == ["daily_countAndRecover", "daily_buildInfectedArray_global",
                       "doWeekday_wholeDay_generateSchedulesKernel", "doWeekday_wholeDay_setup_sort",
                       "doWeekday_wholeDay_setup_locationSearch", "doWeekday_wholeDay_kernel", "doWeekday_wholeDay"]
    assert [r[2] for r in by_day[5]][-1] == "doWeekend_wholeDay"
    assert [r[2] for r in by_day[7]] == ["daily_countAndRecover", "daily_buildInfectedArray_global"]
    # the parent's inclusive time is its children's sum and its exclusive time zero
    kids = sum(float(r[4]) for r in by_day[0][2:6])
    assert abs(float(by_day[0][6][4]) - kids) < 1e-5 and float(by_day[0][6][5]) == 0.0
    assert [int(r[1]) for r in by_day[0]] == [1, 1, 2, 2, 2, 2, 1]
