"""Parity of the CUDA path with the reference (golden vectors made by the reference's own stages)
and with the oracle, through the C ABI of libmhdgb.so.

Tolerances (from the benchmark spec of the FP64 form): relative L-infinity <= 1e-12 after one
step and <= 1e-9 after 100 steps for the FMA-contracted FP64 fused step; bit-for-bit equality
for the stage entry points and for the separately rounded FP64 fused step."""
import numpy as np
import pytest

import oracle as O
from golden_cases import cases
from mhdturbulence_gb300 import MhdgbError, Solver, ic

pytestmark = pytest.mark.gpu
CASES = cases()
GAM = 5.0 / 3.0


def rel_linf(a, b, floor=1e-3):
    """max over fields of max|a-b| / max(max|b|, floor); arrays (nz, ny, nv, nx)."""
    err = 0.0
    for m in range(b.shape[2]):
        scale = max(np.abs(b[:, :, m, :]).max(), floor)
        err = max(err, np.abs(a[:, :, m, :] - b[:, :, m, :]).max() / scale)
    return err


def solver_for(case, precision, quirk=True):
    return Solver(case.nx, case.ny, case.nz, domain=case.domain, bc=case.bc, gam=case.gam,
                  precision=precision, spacing_quirk=quirk)


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_stage_path_bitwise_vs_reference(case):
    with solver_for(case, "fp64_exact") as s:
        s.upload_cons(case.U0())
        s.UpdatePrimitvP()
        assert np.array_equal(case.view(s.download_prim()), case.z["P0"])
        dt, chg = s.stage_step()
        assert dt == case.z["dts"][0] and chg == case.z["chgs"][0]
        assert np.array_equal(case.view(s.download_prim()), case.z["P1"])
        assert np.array_equal(case.view(s.download_cons()), case.z["U1"])
        for n in range(1, case.nsteps):
            dt, chg = s.stage_step()
            assert dt == case.z["dts"][n] and chg == case.z["chgs"][n]
        assert np.array_equal(case.view(s.download_prim()), case.z["PN"])
        assert np.array_equal(case.view(s.download_cons()), case.z["UN"])


def test_stage_fluxes_bitwise_vs_reference():
    case = next(c for c in CASES if c.full)
    with solver_for(case, "fp64_exact") as s:
        s.upload_cons(case.U0())
        s.UpdatePrimitvP()
        s.ControlTimestep()
        s.SetBoundaryCondition()
        s.EvaluateCh()
        for d in (1, 2, 3):
            s.GetNumericalFluxD(d)
            assert np.array_equal(s.download_flux(d), case.z["F1"][d - 1]), f"flux dir {d}"


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_fused_exact_bitwise_vs_reference(case):
    with solver_for(case, "fp64_exact") as s:
        s.upload_cons(case.U0())
        s.step(1)
        r = s.sync()
        assert r.step == 1 and r.dt == case.z["dts"][0] and r.chg == case.z["chgs"][0]
        assert np.array_equal(ic.interior(s.download_cons()), ic.interior(case.z["U1"]) if case.full else case.z["U1"])
        s.step(case.nsteps - 1)
        r = s.sync()
        assert r.step == case.nsteps
        UN = case.z["UN"] if not case.full else ic.interior(case.z["UN"])
        PN = case.z["PN"] if not case.full else ic.interior(case.z["PN"])
        assert np.array_equal(ic.interior(s.download_cons()), UN)
        assert np.array_equal(ic.interior(s.download_prim()), PN)


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_fused_fp64_within_tolerance_of_reference(case):
    with solver_for(case, "fp64") as s:
        s.upload_cons(case.U0())
        s.step(1)
        r = s.sync()
        U1 = case.z["U1"] if not case.full else ic.interior(case.z["U1"])
        assert rel_linf(ic.interior(s.download_cons()), U1) <= 1e-12
        assert abs(r.dt / case.z["dts"][0] - 1) <= 1e-12
        s.step(case.nsteps - 1)
        s.sync()
        UN = case.z["UN"] if not case.full else ic.interior(case.z["UN"])
        assert rel_linf(ic.interior(s.download_cons()), UN) <= 1e-9


def _kh_state(nx, ny, nz, seed=1):
    return ic.prim_to_cons(ic.kh_prim(nx, ny, nz, seed=seed), GAM)


@pytest.mark.parametrize("precision", ["fp64", "fp64_exact"])
def test_fused_vs_oracle_kh_100_steps(precision):
    nx, ny, nz, nsteps = 24, 40, 20, 100
    axes = ic.grid(nx, ny, nz, ic.KH_DOMAIN)
    U0 = _kh_state(nx, ny, nz)
    orc = O.Oracle(nx, ny, nz, *axes, gam=GAM, bc=ic.KH_BC, spacing_quirk=False)
    Uo = U0.copy()
    Po = ic.empty_field(nx, ny, nz, 12)
    orc.update_prim(Uo, Po)
    _, dts1, _ = orc.run(Uo, Po, 1)
    U1o = Uo.copy()
    _, dts, _ = orc.run(Uo, Po, nsteps - 1)
    with Solver(nx, ny, nz, precision=precision) as s:
        s.upload_cons(U0)
        s.step(1)
        r = s.sync()
        e1 = rel_linf(ic.interior(s.download_cons()), ic.interior(U1o))
        s.step(nsteps - 1)
        r = s.sync()
        eN = rel_linf(ic.interior(s.download_cons()), ic.interior(Uo))
        if precision == "fp64_exact":
            assert e1 == 0.0 and eN == 0.0
        assert e1 <= 1e-12, e1
        assert eN <= 1e-9, eN
        assert abs(r.time / (dts1.sum() + dts.sum()) - 1) <= 1e-9
        d = s.diag()
    do = orc.diag(Po)
    assert np.allclose(d, do, rtol=1e-9, atol=0)


def test_mixed_error_vs_fp64():
    nx, ny, nz, nsteps = 32, 64, 16, 60
    U0 = _kh_state(nx, ny, nz, seed=3)
    res = {}
    for prec in ("fp64", "mixed"):
        with Solver(nx, ny, nz, precision=prec) as s:
            s.upload_cons(U0)
            s.step(nsteps)
            res[prec] = (s.sync(), s.download_cons())
    Ud, Um = ic.interior(res["fp64"][1]), ic.interior(res["mixed"][1])
    rho_l1 = np.abs(Um[:, :, 0, :] - Ud[:, :, 0, :]).sum() / np.abs(Ud[:, :, 0, :]).sum()
    assert rho_l1 <= 1e-5, rho_l1
    assert rel_linf(Um, Ud) <= 1e-4
    assert abs(res["mixed"][0].time / res["fp64"][0].time - 1) <= 1e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_conservation_periodic(precision):
    n = 16
    U0 = ic.prim_to_cons(ic.turbulence_prim(n, seed=4), GAM)
    with Solver(n, n, n, domain=ic.CUBE_DOMAIN, bc=ic.PERIODIC_BC, precision=precision) as s:
        s.upload_cons(U0)
        s.step(30)
        s.sync()
        U = ic.interior(s.download_cons())
    U0i = ic.interior(U0)
    for m in (0, 1, 2, 3, 4, 5, 6, 7, 9):  # all but psi (damped)
        tot0, tot = U0i[:, :, m, :].sum(), U[:, :, m, :].sum()
        scale = np.abs(U0i[:, :, m, :]).sum() + 1e-30
        assert abs(tot - tot0) / scale <= (1e-13 if precision == "fp64" else 1e-9), (m, tot, tot0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_run_is_deterministic(precision):
    nx, ny, nz = 40, 24, 36
    U0 = _kh_state(nx, ny, nz, seed=5)
    out = []
    for _ in range(2):
        with Solver(nx, ny, nz, precision=precision) as s:
            s.upload_cons(U0)
            s.step(20)
            s.sync()
            out.append(s.download_cons())
    assert np.array_equal(out[0], out[1])


def test_fused_graph_and_single_launches_agree():
    nx, ny, nz = 20, 20, 20
    U0 = _kh_state(nx, ny, nz, seed=6)
    out = []
    for chunks in ([35], [1] * 35):
        with Solver(nx, ny, nz) as s:
            s.upload_cons(U0)
            for c in chunks:
                s.step(c)
            r = s.sync()
            assert r.step == 35
            out.append(s.download_cons())
    assert np.array_equal(out[0], out[1])


def test_stop_condition_and_run_until():
    nx, ny, nz = 16, 16, 16
    with Solver(nx, ny, nz) as s:
        s.upload_cons(_kh_state(nx, ny, nz))
        r = s.run_until(1e300, max_steps=37)
        assert r.step == 37 and r.done
        s.step(5)  # no-ops after the stop condition
        assert s.sync().step == 37
        s.reset_clock()
        s.upload_cons(_kh_state(nx, ny, nz))
        r = s.run_until(0.05)
        assert r.done and r.time > 0.05 and r.time - r.dt <= 0.05


def test_step_host_matches_resident_steps():
    nx, ny, nz = 16, 24, 12
    U0 = _kh_state(nx, ny, nz, seed=8)
    with Solver(nx, ny, nz) as s:
        Uout = np.zeros_like(U0)
        dt, _ = s.step_host(U0, Uout, 3)
    with Solver(nx, ny, nz) as s:
        s.upload_cons(U0)
        s.step(3)
        r = s.sync()
        assert np.array_equal(ic.interior(Uout), ic.interior(s.download_cons()))
        assert dt == r.dt


def test_nonfinite_state_is_reported():
    # failure detection without a GPU fault: a NaN planted in the host input makes the step's
    # dt/c_h candidates non-finite; the device status word turns that into an error at sync.
    nx, ny, nz = 12, 12, 12
    U0 = _kh_state(nx, ny, nz)
    ic.interior(U0)[3, 4, 4, 5] = np.nan
    with Solver(nx, ny, nz) as s:
        s.upload_cons(U0)
        with pytest.raises(MhdgbError) as ei:
            s.step(1)
            s.sync()
        assert ei.value.code in (-3, -4)


def test_init_kh_matches_python_generator():
    nx, ny, nz = 16, 32, 8
    with Solver(nx, ny, nz) as s:
        s.init_kh(seed=1)
        U = ic.interior(s.download_cons())
    Up = ic.interior(_kh_state(nx, ny, nz, seed=1))
    assert np.allclose(U, Up, rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_exact"])
def test_every_tile_shape_gives_identical_results(precision):
    # the per-cell arithmetic does not depend on the tile shape, so all compiled variants of an FP64
    # form agree bit for bit; an uneven grid exercises partial tiles and chunks.  The mixed form's
    # 2-CTA variants (a 128-register build) contract some FP32 multiply-adds differently from its
    # 1-CTA variants: they agree within 1e-9 relative (the mixed form's own error is ~1e-5).
    nx, ny, nz = 45, 22, 19
    U0 = _kh_state(nx, ny, nz, seed=9)
    outs = []
    with Solver(nx, ny, nz, precision=precision) as s:
        nvar = len(s.variants())
    for v in range(nvar):
        with Solver(nx, ny, nz, precision=precision) as s:
            s.select_variant(v)
            s.upload_cons(U0)
            s.step(7)
            r = s.sync()
            assert r.step == 7
            outs.append(s.download_cons())
    for o in outs[1:]:
        if precision == "mixed":
            assert rel_linf(ic.interior(o), ic.interior(outs[0])) <= 1e-9
        else:
            assert np.array_equal(o, outs[0])
    if precision == "mixed":  # bit for bit within each register build: at most two distinct results
        classes = []
        for o in outs:
            if not any(np.array_equal(o, c) for c in classes):
                classes.append(o)
        assert len(classes) <= 2, len(classes)


def test_autotune_restores_state_and_is_remembered():
    nx, ny, nz = 40, 32, 24
    U0 = _kh_state(nx, ny, nz, seed=10)
    with Solver(nx, ny, nz) as s:
        s.upload_cons(U0)
        s.step(3)
        s.sync()
        ref_state = s.download_cons()
        best = s.autotune(steps=2)
        assert 0 <= best < len(s.variants()) and s.variants()[best][3]
        r = s.sync()
        assert r.step == 3
        assert np.array_equal(s.download_cons(), ref_state)
        s.step(2)
        s.sync()
        after = s.download_cons()
    with Solver(nx, ny, nz) as s2:
        assert s2.variants()[best][3]  # remembered for the same grid and precision
        s2.upload_cons(U0)
        s2.step(5)
        s2.sync()
        assert np.array_equal(s2.download_cons(), after)


def test_state_transfers_round_trip_exactly():
    nx, ny, nz = 13, 9, 7
    rng = np.random.default_rng(0)
    with Solver(nx, ny, nz) as s:
        U = rng.standard_normal((s.ktot, s.jtot, 10, s.itot))
        P = rng.standard_normal((s.ktot, s.jtot, 12, s.itot))
        s.upload_cons(U)
        s.upload_prim(P)
        assert np.array_equal(s.download_cons(), U)
        assert np.array_equal(s.download_prim(), P)


def test_reference_style_upload_of_p_and_u():
    # GenerateProblem fills both P and U (main.cpp:93-183); a P the caller uploads is the one the
    # first stage step uses, even when U is uploaded after it
    case = next(c for c in CASES if c.full)
    with solver_for(case, "fp64_exact") as s:
        s.upload_prim(case.z["P0"])
        s.upload_cons(case.U0())
        dt, chg = s.stage_step()
        assert dt == case.z["dts"][0] and chg == case.z["chgs"][0]
        assert np.array_equal(s.download_cons(), case.z["U1"])


def test_fast_fp64_division_is_within_two_ulp():
    import ctypes as C
    from mhdturbulence_gb300 import _lib
    m = C.c_double()
    assert _lib.lib().mhdgb_selftest_division(0, 1 << 22, 12345, C.byref(m)) == 0
    assert m.value <= 2.0, m.value


def test_per_field_transfers_match_full_arrays():
    nx, ny, nz = 10, 12, 8
    rng = np.random.default_rng(3)
    with Solver(nx, ny, nz) as s:
        U = rng.standard_normal((s.ktot, s.jtot, 10, s.itot))
        s.upload_cons(U)
        import ctypes as C
        L = s._L
        for m in (0, 4, 9):
            a = np.zeros((s.ktot, s.jtot, s.itot))
            assert L.mhdgb_download_cons_field(s._h, m, a.ctypes.data_as(C.POINTER(C.c_double))) == 0
            assert np.array_equal(a, U[:, :, m, :])
        b = rng.standard_normal((s.ktot, s.jtot, s.itot))
        assert L.mhdgb_upload_cons_field(s._h, 3, b.ctypes.data_as(C.POINTER(C.c_double))) == 0
        U[:, :, 3, :] = b
        assert np.array_equal(s.download_cons(), U)
