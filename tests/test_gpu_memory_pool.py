"""Simulations take their device memory from the library's per-GPU pool, which keeps
what they free: creating and destroying simulations of one size reuses the same
memory, and pt_trim_device_memory hands it back to the device."""
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import make_params

pytestmark = pytest.mark.gpu


def test_engines_reuse_pooled_memory_and_trim_returns_it(native_lib):
    torch = pytest.importorskip("torch")
    params = make_params(max_days=20, r_pandemic=1.8, r_seasonal=1.4, initial_pandemic=50, initial_seasonal=50,
                         people_scaling=0.8, location_scaling=0.8)   # about 1.9M persons
    s = pt.PandemicSim(params, 4321)
    s.setupSim()
    first, _ = s.runToCompletion()
    s.close()
    torch.cuda.synchronize()
    free_after_first = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        s = pt.PandemicSim(params, 4321)
        s.setupSim()
        again, _ = s.runToCompletion()
        s.close()
        assert (again == first).all()   # the reused memory holds no state of the last run
    torch.cuda.synchronize()
    # the pool served every later simulation from what the first one freed
    assert torch.cuda.mem_get_info()[0] >= free_after_first - (64 << 20)
    assert native_lib.pt_trim_device_memory() == pt.PT_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] > free_after_first + (100 << 20)
