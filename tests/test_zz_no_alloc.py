"""pt_bucket_table_static: the bucket-table builder that allocates no device memory.

It serves callers that cannot call cudaMalloc on their path (a host that owns all
device memory through its own pool, or a loop whose other streams must not be
stalled by the device-wide synchronisation of cudaMalloc/cudaFree).  Its output must
equal the table the simulation builds for workplaces through the existing entry
points, call after call: the shared scratch keeps the previous call's contents, so a
second call on the same input checks that nothing stale leaks into the result.
This file is collected last so a failure here comes after every other test ran."""
import ctypes

import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import make_params

pytestmark = pytest.mark.gpu


def _bind(lib):
    f = lib.pt_bucket_table_static
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_static_table_equals_setup_workplace_table_twice(native_lib):
    torch = pytest.importorskip("torch")
    build_table = _bind(native_lib)
    sim = pt.PandemicSim(make_params(max_days=5, people_scaling=0.1, location_scaling=0.1), 4242)
    sim.setupSim()
    info = sim.info()
    pop = sim.population()  # the workplace table built by pt_setup
    sim.close()
    N, L = info["number_people"], info["number_workplaces"]
    assert N <= (1 << 20)
    keys = torch.from_numpy(pop["workplace"]).cuda()
    for call in range(2):
        offsets = torch.full((L + 1,), -7, dtype=torch.int32, device="cuda")
        table = torch.full((N,), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = build_table(keys.data_ptr(), N, L, offsets.data_ptr(), table.data_ptr(), None)
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == 0
        if call == 1:  # after the first call has loaded the scratch: no device memory taken
            assert free_after == free_before
        assert np.array_equal(offsets.cpu().numpy(), pop["workplace_offset"])
        assert np.array_equal(table.cpu().numpy(), pop["workplace_people"])


def test_static_table_rejects_oversize_and_bad_keys(native_lib):
    torch = pytest.importorskip("torch")
    build_table = _bind(native_lib)
    keys = torch.zeros(16, dtype=torch.int32, device="cuda")
    out = torch.zeros(16, dtype=torch.int32, device="cuda")
    off = torch.zeros(9, dtype=torch.int32, device="cuda")
    assert build_table(keys.data_ptr(), (1 << 20) + 1, 8, off.data_ptr(), out.data_ptr(), None) == -1
    assert build_table(keys.data_ptr(), 16, (1 << 20) + 1, off.data_ptr(), out.data_ptr(), None) == -1
    keys[3] = 8  # outside [0, 8)
    torch.cuda.synchronize()
    assert build_table(keys.data_ptr(), 16, 8, off.data_ptr(), out.data_ptr(), None) == -1
