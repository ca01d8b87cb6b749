"""The schedule kernels' errand lookup against the reference's form of it, over its
whole input domain.

The reference draws an errand destination by walking the errand types, subtracting
each type's probability while the draw exceeds it, then dividing the remainder by the
probability of the type it stops on with an IEEE division
(device_fishAfterschoolOrErrandDestination_weekday, PandemicSim.cu:2909-2947;
device_fishWeekendErrandDestination, :1017-1044).  The kernels run the subtraction
chain to the end and select the stop (no branches), and divide by multiplying with
the rounded reciprocal plus one correction step (Markstein).  The self-test compares
the two on every one of the 2^32 random words a schedule can draw, and the division
on 0 and every float in [2^-32, 1] (the values the search divides) for every
probability the search can stop on."""
import ctypes

import pytest

import pandemicthrust_gb300 as pt

pytestmark = pytest.mark.gpu


def test_errand_lookup_equals_the_loop_and_division_on_every_input(native_lib):
    f = native_lib.pt_selftest_errand_lookup
    f.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
    f.restype = ctypes.c_int
    counts = (ctypes.c_uint64 * 4)(1, 1, 1, 1)
    assert f(counts) == pt.PT_OK
    assert list(counts) == [0, 0, 0, 0], dict(zip(["weekday", "weekend", "division", "reciprocal"], counts))
