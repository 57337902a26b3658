"""HLLE and HLLC (src_f90_acc_device/mhd.f90:877-1141) on the GPU paths against the oracle's
restatement: bit for bit for the stage entry points and the separately rounded fused step; the
FP64 fused step within the FP64 form's tolerance (1e-12 after one step, 1e-9 after many); the
mixed form's density error against FP64 within 1e-5; ensembles with a solver per member."""
import numpy as np
import pytest

import oracle as O
from mhdturbulence_gb300 import Ensemble, MhdgbError, Solver, ic

pytestmark = pytest.mark.gpu
GAM = 5.0 / 3.0
SOLVERS = {"hlle": 1, "hllc": 2}
NX, NY, NZ = 10, 20, 12   # spacing_quirk needs nx <= ny, nz


def rel_linf(a, b, floor=1e-3):
    err = 0.0
    for m in range(b.shape[2]):
        scale = max(np.abs(b[:, :, m, :]).max(), floor)
        err = max(err, np.abs(a[:, :, m, :] - b[:, :, m, :]).max() / scale)
    return err


def oracle_run(U0, nsteps, riemann, quirk):
    orc = O.Oracle(NX, NY, NZ, *ic.grid(NX, NY, NZ), gam=GAM, bc=ic.KH_BC, spacing_quirk=quirk, riemann=riemann)
    U = U0.copy()
    P = ic.empty_field(NX, NY, NZ, 12)
    orc.update_prim(U, P)
    _, dts, chgs = orc.run(U, P, nsteps)
    return U, P, dts, chgs


def kh_state(seed=2):
    return ic.prim_to_cons(ic.kh_prim(NX, NY, NZ, seed=seed, amp=0.05, noise=1e-2), GAM)


@pytest.mark.parametrize("name", list(SOLVERS))
def test_stage_path_bitwise_vs_oracle(name):
    U0 = kh_state()
    Uo, Po, dts, chgs = oracle_run(U0, 4, SOLVERS[name], quirk=True)
    with Solver(NX, NY, NZ, precision="fp64_exact", spacing_quirk=True, riemann=name) as s:
        assert s.riemann == name
        s.upload_cons(U0)
        s.UpdatePrimitvP()
        for n in range(4):
            dt, chg = s.stage_step()
            assert dt == dts[n] and chg == chgs[n]
        assert np.array_equal(ic.interior(s.download_cons()), ic.interior(Uo))
        assert np.array_equal(ic.interior(s.download_prim()), ic.interior(Po))


@pytest.mark.parametrize("name", list(SOLVERS))
def test_fused_exact_bitwise_and_fp64_within_tolerance(name):
    U0 = kh_state(seed=3)
    U1, _, _, _ = oracle_run(U0, 1, SOLVERS[name], quirk=False)
    UN, _, dts, _ = oracle_run(U0, 40, SOLVERS[name], quirk=False)
    for prec in ("fp64_exact", "fp64"):
        with Solver(NX, NY, NZ, precision=prec, riemann=name) as s:
            s.upload_cons(U0)
            s.step(1)
            s.sync()
            e1 = rel_linf(ic.interior(s.download_cons()), ic.interior(U1))
            s.step(39)
            r = s.sync()
            eN = rel_linf(ic.interior(s.download_cons()), ic.interior(UN))
        if prec == "fp64_exact":
            assert e1 == 0.0 and eN == 0.0
            assert r.time == dts.sum() or abs(r.time / dts.sum() - 1) < 1e-15
        assert e1 <= 1e-12 and eN <= 1e-9, (prec, e1, eN)


@pytest.mark.parametrize("name", list(SOLVERS))
def test_mixed_error_and_conservation(name):
    n = 16
    U0 = ic.prim_to_cons(ic.random_smooth_prim(n, n, n, seed=8), GAM)
    res = {}
    for prec in ("fp64", "mixed"):
        with Solver(n, n, n, domain=ic.CUBE_DOMAIN, bc=ic.PERIODIC_BC, precision=prec, riemann=name) as s:
            s.upload_cons(U0)
            s.step(30)
            s.sync()
            res[prec] = ic.interior(s.download_cons())
    Ud, Um = res["fp64"], res["mixed"]
    assert np.abs(Um[:, :, 0, :] - Ud[:, :, 0, :]).sum() / np.abs(Ud[:, :, 0, :]).sum() <= 1e-5
    U0i = ic.interior(U0)
    for U, tol in ((Ud, 1e-13), (Um, 1e-9)):
        assert abs(U[:, :, 0, :].sum() / U0i[:, :, 0, :].sum() - 1) < tol
        assert abs(U[:, :, 4, :].sum() / U0i[:, :, 4, :].sum() - 1) < tol


def test_ensemble_members_with_their_own_solvers():
    specs = [dict(nx=NX, ny=NY, nz=NZ), dict(nx=16, ny=12, nz=8), dict(nx=NX, ny=NY, nz=NZ)]
    states = [ic.prim_to_cons(ic.kh_prim(sp["nx"], sp["ny"], sp["nz"], seed=i + 1), GAM) for i, sp in enumerate(specs)]
    names = ["hlld", "hlle", "hllc"]
    with Ensemble(specs, precision="fp64") as ens:
        for m, U, nm in zip(ens.members, states, names):
            m.upload_cons(U)
        ens.step(5)
        ens.sync()
        for m, nm in zip(ens.members, names):   # change after the first steps: descriptors refresh
            m.set_riemann(nm)
        ens.step(6)
        ens.sync()
        got = [m.download_cons() for m in ens.members]
    # With an HLLE/HLLC member the whole ensemble runs on the run-time solver kernel; its HLLD member
    # then agrees with the HLLD-only kernels of a single run within the FP64 tolerance, the HLLE and
    # HLLC members (the same kernel in both runs) bit for bit.
    for sp, U, nm, g in zip(specs, states, names, got):
        with Solver(sp["nx"], sp["ny"], sp["nz"], precision="fp64") as s:
            s.upload_cons(U)
            s.step(5)
            s.sync()
            s.set_riemann(nm)
            s.step(6)
            s.sync()
            mine = ic.interior(s.download_cons())
        if nm == "hlld":
            assert rel_linf(ic.interior(g), mine) <= 1e-12, nm
        else:
            assert np.array_equal(mine, ic.interior(g)), nm


def test_unknown_solver_is_refused():
    with Solver(8, 8, 8) as s:
        with pytest.raises(MhdgbError):
            s._ck(s._L.mhdgb_set_riemann(s._h, 3), "set_riemann")
        assert s.riemann == "hlld"
