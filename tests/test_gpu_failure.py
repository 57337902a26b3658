"""Failure detection on the GPU without a fault.  A device-side wait that nothing completes gives up
at its time limit and reports a status the host reads; the context stays usable afterwards."""
import ctypes as C

import pytest

from mhdturbulence_gb300 import Solver, _lib

pytestmark = pytest.mark.gpu
ST_TIMEOUT = 4


def test_bounded_wait_gives_up_and_reports_a_status():
    seconds, status = C.c_double(), C.c_uint()
    assert _lib.lib().mhdgb_selftest_wait_timeout(0, C.byref(seconds), C.byref(status)) == 0
    assert status.value & ST_TIMEOUT
    assert 1.0 <= seconds.value <= 30.0, seconds.value
    # the context is intact: a solver steps normally in the same process afterwards
    with Solver(16, 16, 16) as s:
        s.init_kh(seed=1)
        s.step(3)
        r = s.sync()
        assert r.status == 0 and r.step == 3
