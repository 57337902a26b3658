"""Checkpoint / restart: a run restarted from a checkpoint continues bit for bit (same precision),
the file carries the state and clock, and mismatched or damaged files are refused."""
import numpy as np
import pytest

from mhdturbulence_gb300 import MhdgbError, Solver, ic

pytestmark = pytest.mark.gpu
NX, NY, NZ = 20, 24, 12


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_exact"])
def test_restart_continues_bit_for_bit(tmp_path, precision):
    ck = str(tmp_path / "state.ck")
    with Solver(NX, NY, NZ, precision=precision) as s:
        s.init_kh(seed=5)
        s.set_stop(1e300, 1000)
        s.step(9)
        r0 = s.sync()
        s.checkpoint_save(ck)
        s.step(21)
        ra = s.sync()
        Ua = s.download_cons()
    with Solver(NX, NY, NZ, precision=precision) as s:
        s.checkpoint_load(ck)
        r1 = s.sync()
        assert (r1.step, r1.time, r1.dt, r1.chg) == (r0.step, r0.time, r0.dt, r0.chg)
        s.step(21)
        rb = s.sync()
        Ub = s.download_cons()
    assert (rb.step, rb.time, rb.dt, rb.chg) == (ra.step, ra.time, ra.dt, ra.chg)
    assert np.array_equal(ic.interior(Ub), ic.interior(Ua))


def test_restart_keeps_physics_and_stop(tmp_path):
    ck = str(tmp_path / "s.ck")
    bc = (ic.BC_OUTFLOW, ic.BC_OUTFLOW, ic.BC_REFLECTION, ic.BC_REFLECTION, ic.BC_PERIODIC, ic.BC_PERIODIC)
    with Solver(NX, NY, NZ, bc=bc, gam=1.4, cfl=0.1) as s:
        s.init_kh(seed=2)
        s.set_stop(1e300, 12)
        s.step(5)
        s.sync()
        s.checkpoint_save(ck)
        s.step(20)                   # stops at step 12
        ra = s.sync()
        Ua = s.download_cons()
    with Solver(NX, NY, NZ) as s:    # default gam, cfl and boundaries: the checkpoint's replace them
        s.checkpoint_load(ck)
        s.step(20)
        rb = s.sync()
        assert rb.done and rb.step == 12
        assert (rb.time, rb.dt) == (ra.time, ra.dt)
        assert np.array_equal(s.download_cons(), Ua)


def test_bad_checkpoints_are_refused(tmp_path):
    ck = tmp_path / "s.ck"
    with Solver(NX, NY, NZ) as s:
        s.init_kh()
        s.checkpoint_save(str(ck))
    with Solver(NX + 1, NY, NZ) as s:
        with pytest.raises(MhdgbError) as e:
            s.checkpoint_load(str(ck))
        assert e.value.code == -1
    bad = tmp_path / "bad.ck"
    bad.write_bytes(b"not a checkpoint at all")
    short = tmp_path / "short.ck"
    short.write_bytes(ck.read_bytes()[:1000])
    with Solver(NX, NY, NZ) as s:
        for path, code in ((bad, -1), (short, -9), (tmp_path / "missing.ck", -9)):
            with pytest.raises(MhdgbError) as e:
                s.checkpoint_load(str(path))
            assert e.value.code == code
        s.init_kh()
        s.step(2)
        assert s.sync().step == 2    # the handle stays usable
