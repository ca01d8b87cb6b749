"""The drop-in executable: constants.csv + seed.txt in a directory produce the
reference's output files, byte-identical to the oracle's."""
import os
import subprocess

import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import make_params, oracle_run_to_files, write_inputs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("params,seed,flags", [
    (make_params(max_days=30, r_pandemic=1.4, r_seasonal=1.2, initial_pandemic=10, initial_seasonal=10,
                 people_scaling=0.04248, location_scaling=0.04248), 12345, []),
    (make_params(max_days=120, people_scaling=0.02, location_scaling=0.02, percent_symptomatic=0.5,
                 asymp_factor=0.5), 2024, ["--per-day"]),
    (make_params(max_days=50, people_scaling=0.01, location_scaling=0.01, initial_pandemic=0,
                 initial_seasonal=0), 9, []),
])
def test_cli_outputs_match_oracle(native_lib, oracle_built, tmp_path, params, seed, flags):
    gdir = tmp_path / "gpu"
    odir = tmp_path / "oracle"
    gdir.mkdir()
    odir.mkdir()
    write_inputs(str(gdir), params, seed)
    proc = subprocess.run([pt.CLI_PATH] + flags, cwd=str(gdir), capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    assert "people" in proc.stdout and "seeds:" in proc.stdout
    oracle_run_to_files(params, seed, str(odir))
    for name in ("output_infected_stats.csv", "output_rn.csv", "infected_max.txt"):
        assert (gdir / name).read_bytes() == (odir / name).read_bytes(), name
    assert (gdir / "output_resource_log.csv").exists()


def test_cli_missing_inputs_fail_like_reference(native_lib, tmp_path):
    proc = subprocess.run([pt.CLI_PATH], cwd=str(tmp_path), capture_output=True, text=True, timeout=60)
    assert proc.returncode == 1
    assert "Error opening seed file" in proc.stderr


PROFILE_NAMES = {"setupSim", "daily_countAndRecover", "daily_buildInfectedArray_global",
                 "doWeekday_wholeDay_generateSchedulesKernel", "doWeekday_wholeDay_setup_sort",
                 "doWeekday_wholeDay_setup_locationSearch", "doWeekday_wholeDay_kernel", "doWeekday_wholeDay",
                 "weekend_assignErrands", "doWeekend_wholeDay_setup_sort", "doWeekend_wholeDay_setup_locationSearch",
                 "doWeekend_wholeDay_kernel", "doWeekend_wholeDay", "final_countReproduction", "runToCompletion"}


def test_cli_profile_and_memory_logs_in_reference_format(native_lib, tmp_path):
    # profiler.cu:13 (header) and :72-76 (row format "%d, %d, %s, %d, %f, %lf");
    # resource_logging.cu:47-51, :73-78 (output_mem.csv)
    params = make_params(max_days=20, r_pandemic=1.6, r_seasonal=1.3, initial_pandemic=10, initial_seasonal=10,
                         people_scaling=0.02, location_scaling=0.02)
    write_inputs(str(tmp_path), params, 77)
    proc = subprocess.run([pt.CLI_PATH, "--quiet", "--mem-log"], cwd=str(tmp_path), capture_output=True, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stderr
    lines = (tmp_path / "profile_log.csv").read_text().splitlines()
    assert lines[0] == ("day,stack_depth,function_name,problem_size,inclusive_time_milliseconds,"
                        "exclusive_time_milliseconds")
    days = set()
    for row in lines[1:]:
        f = row.split(", ")
        assert len(f) == 6, row
        day, depth, name, size = int(f[0]), int(f[1]), f[2], int(f[3])
        incl, excl = float(f[4]), float(f[5])
        assert name in PROFILE_NAMES and 0 <= depth <= 2 and size >= 0 and incl >= 0 and excl >= 0, row
        assert len(f[4].split(".")[1]) == 6  # %f
        if name == "daily_countAndRecover":
            days.add(day)
    rows = len((tmp_path / "output_infected_stats.csv").read_text().splitlines()) - 1
    assert days == set(range(rows))
    mem = (tmp_path / "output_mem.csv").read_text().splitlines()
    assert mem[0] == "day,freeBytes,bytesUsed,totalBytes,megabytesUsed"
    assert mem[1].startswith("INITIAL,") and mem[1].split(",")[2] == "0"
    assert len(mem) == 2 + rows and all(len(r.split(",")) == 5 for r in mem)
    # --no-profile: no profile log, same results
    (tmp_path / "profile_log.csv").unlink()
    before = (tmp_path / "output_infected_stats.csv").read_bytes()
    proc = subprocess.run([pt.CLI_PATH, "--quiet", "--no-profile"], cwd=str(tmp_path), capture_output=True,
                          text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    assert not (tmp_path / "profile_log.csv").exists()
    assert (tmp_path / "output_infected_stats.csv").read_bytes() == before


def _write_experiments(root):
    # the layout PythonBatcher/write_gpu_constants.py writes: one directory per
    # experiment with its constants.csv, and experiment_files.txt listing them
    exps = {
        "p0.02_l0.02_10_10": make_params(max_days=30, r_pandemic=1.8, r_seasonal=1.3, initial_pandemic=10,
                                         initial_seasonal=10, people_scaling=0.02, location_scaling=0.02),
        "p0.01_l0.1_30_5": make_params(max_days=40, r_pandemic=1.4, r_seasonal=1.9, initial_pandemic=30,
                                       initial_seasonal=5, people_scaling=0.01, location_scaling=0.1),
        "p0.005_l0.005_3_3": make_params(max_days=25, r_pandemic=0.6, r_seasonal=0.5, initial_pandemic=3,
                                         initial_seasonal=3, people_scaling=0.005, location_scaling=0.005),
    }
    base = root / "gpu_experiment_files"
    base.mkdir()
    listing = []
    for name, p in exps.items():
        d = base / name
        d.mkdir()
        write_inputs(str(d), p, 0)
        (d / "seed.txt").unlink()
        listing.append(str(d / "constants.csv"))
    (base / "experiment_files.txt").write_text("\n".join(listing) + "\n")
    return base, exps


def _alone(tmp_path, params, seed, tag):
    d = tmp_path / ("alone_" + tag)
    d.mkdir()
    write_inputs(str(d), params, seed)
    proc = subprocess.run([pt.CLI_PATH, "--quiet", "--no-profile"], cwd=str(d), capture_output=True, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stderr
    return d


def test_batch_driver_runs_a_scenario_grid_like_separate_runs(native_lib, tmp_path):
    base, exps = _write_experiments(tmp_path)
    proc = subprocess.run([pt.BATCH_CLI_PATH, "--list", str(base / "experiment_files.txt"), "--seeds", "11,12"],
                          cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    assert len(proc.stdout.splitlines()) == 2 * len(exps)
    for name, p in exps.items():
        for seed in (11, 12):
            out = base / name / ("seed_%d" % seed)
            ref = _alone(tmp_path, p, seed, "%s_%d" % (name, seed))
            for f in ("output_infected_stats.csv", "output_rn.csv", "infected_max.txt"):
                assert (out / f).read_bytes() == (ref / f).read_bytes(), (name, seed, f)
            assert (out / "output_resource_log.csv").read_text().splitlines()[1].startswith("gb300_native_batch,")


def test_batch_driver_reads_each_experiments_seed_file(native_lib, tmp_path):
    base, exps = _write_experiments(tmp_path)
    for i, name in enumerate(exps):
        (base / name / "seed.txt").write_text("%d\n" % (500 + i))
    proc = subprocess.run([pt.BATCH_CLI_PATH, "--list", str(base / "experiment_files.txt"), "--quiet"],
                          cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    for i, (name, p) in enumerate(exps.items()):
        ref = _alone(tmp_path, p, 500 + i, name)
        for f in ("output_infected_stats.csv", "output_rn.csv", "infected_max.txt"):
            assert (base / name / f).read_bytes() == (ref / f).read_bytes(), (name, f)
    # a missing list fails like a missing input file
    proc = subprocess.run([pt.BATCH_CLI_PATH, "--list", str(tmp_path / "nope.txt")], cwd=str(tmp_path),
                          capture_output=True, text=True, timeout=60)
    assert proc.returncode == 1
