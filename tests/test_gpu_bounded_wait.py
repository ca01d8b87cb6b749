"""A device-side wait that runs out returns PT_ERR_TIMEOUT and leaves the GPU usable.

Every wait of one thread block for another (the decoupled look-backs of the scans and
sorts) is bounded.  pt_selftest_bounded_wait runs that wait code in one small kernel
whose predecessor never publishes (a flag that nothing sets): the wait gives up after
the given number of polls, the kernel records its error word and ends normally.  No
GPU fault, trap or hang is involved.  The reference never checks kernel errors
(PandemicSim.cu:2754-2761)."""
import ctypes

import numpy as np
import pytest

import pandemicthrust_gb300 as pt
from oracle.oracle import Oracle, make_params

pytestmark = pytest.mark.gpu


def _probe(lib):
    f = lib.pt_selftest_bounded_wait
    f.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint32)]
    f.restype = ctypes.c_int
    return f


def test_wait_with_a_published_predecessor_returns_its_prefix(native_lib):
    probe = _probe(native_lib)
    prefix = ctypes.c_uint32(0)
    assert probe(1, 1 << 20, ctypes.byref(prefix)) == pt.PT_OK
    assert prefix.value == 1234


@pytest.mark.parametrize("limit", [0, 1000, 1 << 16])
def test_wait_that_runs_out_reports_timeout_and_the_device_stays_usable(native_lib, oracle_built, limit):
    probe = _probe(native_lib)
    prefix = ctypes.c_uint32(7)
    assert probe(0, limit, ctypes.byref(prefix)) == pt.PT_ERR_TIMEOUT
    assert b"gave up" in native_lib.pt_last_error(None)
    # the context is intact: a simulation still runs and still equals the oracle
    p = make_params(max_days=10, people_scaling=0.01, location_scaling=0.01, r_pandemic=2.0)
    sim = pt.PandemicSim(p, 17)
    sim.setupSim()
    counts, infected = sim.runToCompletion()
    st = sim.person_state()
    sim.close()
    o = Oracle(p, 17)
    o.setup()
    for d in range(len(infected)):
        rc, c, i = o.step_day()
        assert c == counts[d].tolist() and i == infected[d], d
    v = o.view()
    for k in ("status_p", "status_s", "gen_p", "gen_s"):
        assert np.array_equal(st[k], v[k]), k
    o.close()


def test_spin_limit_outside_the_range_is_rejected(native_lib):
    probe = _probe(native_lib)
    assert probe(0, -1, None) == pt.PT_ERR_ARG
    assert probe(0, (1 << 22) + 1, None) == pt.PT_ERR_ARG
