"""Failure detection on the GPU without a fault.  A device-side wait that nothing completes gives up
at its time limit and reports a status the host reads; the context stays usable afterwards.  Both
the standalone bounded wait and the fused step's own abort-and-drain path are made to run."""
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


@pytest.mark.parametrize("precision", [0, 2], ids=["fp64", "mixed"])
def test_fused_step_aborts_drains_and_recovers(precision):
    """The fused step's own abort path: a plane load that never completes its barrier makes every
    CTA give up its bounded wait, drain and return; the step reports the timeout bit, and the same
    handle then steps bit for bit like one that never saw the aborted step."""
    seconds, status, recovered = C.c_double(), C.c_uint(), C.c_int()
    rc = _lib.lib().mhdgb_selftest_fused_abort(0, precision, C.byref(seconds), C.byref(status),
                                                C.byref(recovered))
    assert rc == 0, _lib.STATUS.get(rc, rc)
    assert status.value & ST_TIMEOUT
    assert 1.0 <= seconds.value <= 30.0, seconds.value
    assert recovered.value == 1
