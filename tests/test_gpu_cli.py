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
