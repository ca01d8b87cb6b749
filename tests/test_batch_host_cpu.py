"""Host side of the batch API that needs no GPU: argument checks, per-instance
parameter validation, and each instance's seeds and scaling equal to the same
simulation created alone."""
import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import make_params


def test_batch_rejects_bad_instance_counts(native_lib):
    with pytest.raises(ValueError):
        pt.PandemicBatch([make_params()], [1, 2])
    with pytest.raises(pt.PtError) as e:
        pt.PandemicBatch([], [])
    assert e.value.code == -1
    with pytest.raises(pt.PtError) as e:
        pt.PandemicBatch([make_params()] * 4097, list(range(4097)))
    assert e.value.code == -1


def test_batch_names_the_invalid_instance(native_lib):
    params = [make_params() for _ in range(4)]
    params[2]["max_days"] = 300
    with pytest.raises(pt.PtError) as e:
        pt.PandemicBatch(params, [1, 2, 3, 4])
    assert e.value.code == -1 and "instance 2" in str(e.value)


def test_batch_instances_derive_like_standalone(native_lib):
    params = [make_params(people_scaling=0.04248, location_scaling=0.04248),
              make_params(people_scaling=0.5, location_scaling=1.5, r_pandemic=1.9, r_seasonal=1.1),
              make_params(percent_symptomatic=0.6, asymp_factor=0.3, max_days=12)]
    seeds = [12345, 1003, -5]
    b = pt.PandemicBatch(params, seeds)
    assert b.size() == (3, 0, 0)  # persons are known after setup
    for k, (p, s) in enumerate(zip(params, seeds)):
        bi = b.info(k)
        sim = pt.PandemicSim(p, s)
        si = sim.info()
        for key in ("seeds", "number_households", "number_workplaces", "type_count", "type_offset"):
            assert bi[key] == si[key], (k, key)
        assert np.array(bi["infectiousness"], np.float32).tobytes() == np.array(si["infectiousness"], np.float32).tobytes()
        sim.close()
    b.close()


def test_batch_driver_rejects_bad_arguments_before_any_device_work(native_lib, tmp_path):
    import subprocess
    proc = subprocess.run([pt.BATCH_CLI_PATH, "--list", str(tmp_path / "missing.txt")], cwd=str(tmp_path),
                          capture_output=True, text=True, timeout=60)
    assert proc.returncode == 1 and "missing.txt" in proc.stderr
    proc = subprocess.run([pt.BATCH_CLI_PATH, "--seeds", "1,,2"], cwd=str(tmp_path), capture_output=True, text=True,
                          timeout=60)
    assert proc.returncode == 2
    (tmp_path / "empty.txt").write_text("\n")
    proc = subprocess.run([pt.BATCH_CLI_PATH, "--list", str(tmp_path / "empty.txt")], cwd=str(tmp_path),
                          capture_output=True, text=True, timeout=60)
    assert proc.returncode == 1 and "no experiments" in proc.stderr
