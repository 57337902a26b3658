"""The stated workloads at their stated sizes.  KH on 64^3 for 100 steps and on the 150^3 benchmark
grid is checked against the oracle directly (the oracle steps 150^3 in a fraction of a second on the
host's cores).  Decaying
turbulence on a periodic 256^3 cube is checked through properties that hold at any size:
conservation to round-off, and the mixed form's distance from FP64.  KH at 512^3 is checked
through reruns that must be identical, and the mixed form's KH diagnostic against FP64's.  At
512^3 a state is 11 GB, so only reports and diagnostics come back to the host."""
import numpy as np
import pytest

import oracle as O
from mhdturbulence_gb300 import Solver, ic

pytestmark = pytest.mark.gpu
GAM = 5.0 / 3.0


def rel_linf(a, b, floor=1e-3):
    """max over fields of max|a-b| / max(max|b|, floor); arrays (nz, ny, nv, nx)."""
    err = 0.0
    for m in range(b.shape[2]):
        scale = max(np.abs(b[:, :, m, :]).max(), floor)
        err = max(err, np.abs(a[:, :, m, :] - b[:, :, m, :]).max() / scale)
    return err


@pytest.mark.parametrize("cfl", [0.05, 0.3], ids=["cfl0.05", "cfl0.3"])
def test_kh_64_100_steps_vs_oracle(cfl):
    """The small plain-method configuration as stated: KH on 64^3 cells, FP64, gamma = 5/3, 100 steps
    against the oracle (equal bit for bit to the reference's CPU stages), at the reference's CFL
    factor 0.05 (mhd.cpp:1560) and at the stated 0.3.  FMA-contracted FP64: relative L-inf <= 1e-12
    after 1 step and <= 1e-9 after 100; separately rounded FP64: bit for bit, every step's dt too;
    the KH diagnostic (volume, mixing, sqrt(<v_y^2>)) within 1e-9 of the oracle's."""
    n, nsteps = 64, 100
    U0 = ic.prim_to_cons(ic.kh_prim(n, n, n, seed=1), GAM)
    orc = O.Oracle(n, n, n, *ic.grid(n, n, n, ic.KH_DOMAIN), gam=GAM, cfl=cfl, bc=ic.KH_BC, spacing_quirk=False)
    Uo, Po = U0.copy(), ic.empty_field(n, n, n, 12)
    orc.update_prim(Uo, Po)
    _, dts1, chg1 = orc.run(Uo, Po, 1)
    U1o = ic.interior(Uo).copy()
    _, dts, chgs = orc.run(Uo, Po, nsteps - 1)
    UNo, PNo = ic.interior(Uo), ic.interior(Po)
    diag_o = orc.diag(Po)
    tsum = dts1.sum() + dts.sum()
    for precision, tol1, tol_n in (("fp64", 1e-12, 1e-9), ("fp64_exact", 0.0, 0.0)):
        with Solver(n, n, n, precision=precision, cfl=cfl) as s:
            s.upload_cons(U0)
            s.step(1)
            r = s.sync()
            assert rel_linf(ic.interior(s.download_cons()), U1o) <= tol1, precision
            assert abs(r.dt / dts1[0] - 1) <= tol1 and abs(r.chg / chg1[0] - 1) <= tol1, precision
            for q in range(nsteps - 1):  # every step's dt and c_h
                s.step(1)
                r = s.sync()
                assert abs(r.dt / dts[q] - 1) <= max(tol_n, 1e-12 if tol_n else 0.0), (precision, q)
                assert abs(r.chg / chgs[q] - 1) <= max(tol_n, 1e-12 if tol_n else 0.0), (precision, q)
            assert r.step == nsteps
            assert rel_linf(ic.interior(s.download_cons()), UNo) <= tol_n, precision
            if precision == "fp64_exact":
                assert np.array_equal(ic.interior(s.download_prim()), PNo)
                assert r.time == tsum
            assert abs(r.time / tsum - 1) <= 1e-12
            assert np.allclose(s.diag(), diag_o, rtol=1e-9, atol=0), precision


def test_kh_150_benchmark_grid_vs_oracle():
    n, nsteps = 150, 3
    U0 = ic.prim_to_cons(ic.kh_prim(n, n, n, seed=1), GAM)
    orc = O.Oracle(n, n, n, *ic.grid(n, n, n, ic.KH_DOMAIN), gam=GAM, bc=ic.KH_BC, spacing_quirk=False)
    Uo, Po = U0.copy(), ic.empty_field(n, n, n, 12)
    orc.update_prim(Uo, Po)
    _, dts1, _ = orc.run(Uo, Po, 1)
    U1o = ic.interior(Uo).copy()
    _, dts, _ = orc.run(Uo, Po, nsteps - 1)
    UNo = ic.interior(Uo)
    # FMA-contracted FP64 form: the tolerances of the FP64 form; separately rounded form: bit for bit
    for precision, tol1, tol_n in (("fp64", 1e-12, 1e-11), ("fp64_exact", 0.0, 0.0)):
        with Solver(n, n, n, precision=precision) as s:
            s.upload_cons(U0)
            s.step(1)
            r = s.sync()
            e1 = rel_linf(ic.interior(s.download_cons()), U1o)
            assert e1 <= tol1, (precision, e1)
            assert abs(r.dt / dts1[0] - 1) <= max(tol1, 0.0), precision
            s.step(nsteps - 1)
            r = s.sync()
            e_n = rel_linf(ic.interior(s.download_cons()), UNo)
            assert e_n <= tol_n, (precision, e_n)
            assert abs(r.time / (dts1.sum() + dts.sum()) - 1) <= 1e-12


@pytest.fixture(scope="module")
def turb256():
    """The seeded decaying-turbulence state on the periodic 256^3 cube (log-normal density with
    sigma_ln_rho = 0.3, k^-2 velocity and vector-potential spectra over 1 <= |k| <= 8, v_rms = 0.5,
    mean B_x = 0.2, beta = 10, p = 1)."""
    return ic.prim_to_cons(ic.turbulence_prim(256, seed=4), GAM)


def _divb_rms_periodic(U, axes):
    """rms of the central-difference divergence of B over a periodic box; U interior (nz, ny, nv, nx)."""
    dx, dy, dz = (np.diff(a)[2:2 + n] for a, n in zip(axes, (U.shape[3], U.shape[1], U.shape[0])))
    bx, by, bz = U[:, :, 5, :], U[:, :, 6, :], U[:, :, 7, :]
    d = (np.roll(bx, -1, 2) - np.roll(bx, 1, 2)) / (2 * dx[None, None, :]) \
        + (np.roll(by, -1, 1) - np.roll(by, 1, 1)) / (2 * dy[None, :, None]) \
        + (np.roll(bz, -1, 0) - np.roll(bz, 1, 0)) / (2 * dz[:, None, None])
    return float(np.sqrt(np.mean(d ** 2)))


def test_turbulence_256_200_steps_mixed_vs_fp64(turb256):
    """The stated mixed-precision configuration: 200 steps of the 256^3 turbulence state in the mixed
    form and in FP64.  Bound: density L1 relative error <= 1e-5 against FP64 (the task's bound for the
    mixed form).  Density L-inf, total-energy density L1 and the divergence of B are held to the
    margins measured for this state (each about 10x above what was measured), and both forms
    conserve mass, momentum, energy, field and tracer."""
    n, nsteps = 256, 200
    axes = ic.grid(n, n, n, ic.CUBE_DOMAIN)
    out, reps = {}, {}
    for precision in ("fp64", "mixed"):
        with Solver(n, n, n, domain=ic.CUBE_DOMAIN, bc=ic.PERIODIC_BC, precision=precision) as s:
            s.upload_cons(turb256)
            s.step(nsteps)
            r = s.sync()
            assert r.step == nsteps and r.status == 0
            out[precision], reps[precision] = ic.interior(s.download_cons()), r
    Uf, Um = out["fp64"], out["mixed"]
    rho_f, rho_m = Uf[:, :, 0, :], Um[:, :, 0, :]
    rho_l1 = np.abs(rho_m - rho_f).sum() / np.abs(rho_f).sum()
    rho_linf = np.abs(rho_m - rho_f).max() / np.abs(rho_f).max()
    e_l1 = np.abs(Um[:, :, 4, :] - Uf[:, :, 4, :]).sum() / np.abs(Uf[:, :, 4, :]).sum()
    div0, divf, divm = (_divb_rms_periodic(U, axes) for U in (ic.interior(turb256), Uf, Um))
    print(f"turbulence 256^3 x {nsteps}: rho L1 {rho_l1:.3e}, rho Linf {rho_linf:.3e}, energy L1 {e_l1:.3e}, "
          f"divB rms initial {div0:.6e} fp64 {divf:.6e} mixed {divm:.6e}, time {reps['fp64'].time:.6e} "
          f"vs {reps['mixed'].time:.6e}")
    assert rho_l1 <= 1e-5, rho_l1
    assert rho_linf <= 2e-5, rho_linf
    assert e_l1 <= 2e-7, e_l1
    assert abs(divm / divf - 1) <= 1e-6, (divm, divf)
    assert abs(reps["mixed"].time / reps["fp64"].time - 1) <= 1e-6
    U0i = ic.interior(turb256)
    for precision, tol in (("fp64", 1e-13), ("mixed", 1e-9)):
        for m in (0, 1, 2, 3, 4, 5, 6, 7, 9):  # all but psi (damped)
            tot0, tot = U0i[:, :, m, :].sum(), out[precision][:, :, m, :].sum()
            scale = np.abs(U0i[:, :, m, :]).sum() + 1e-30
            assert abs(tot - tot0) / scale <= tol, (precision, m, tot, tot0)


def test_turbulence_256_conserves_and_mixed_tracks_fp64(turb256):
    n, nsteps = 256, 10
    U0 = turb256
    out = {}
    for precision in ("fp64", "mixed"):
        with Solver(n, n, n, domain=ic.CUBE_DOMAIN, bc=ic.PERIODIC_BC, precision=precision) as s:
            s.upload_cons(U0)
            s.step(nsteps)
            r = s.sync()
            assert r.step == nsteps and r.status == 0
            out[precision] = ic.interior(s.download_cons())
    U0i = ic.interior(U0)
    for precision, tol in (("fp64", 1e-13), ("mixed", 1e-9)):
        U = out[precision]
        for m in (0, 1, 2, 3, 4, 5, 6, 7, 9):  # all but psi (damped)
            tot0, tot = U0i[:, :, m, :].sum(), U[:, :, m, :].sum()
            scale = np.abs(U0i[:, :, m, :]).sum() + 1e-30
            assert abs(tot - tot0) / scale <= tol, (precision, m, tot, tot0)
    rho_f, rho_m = out["fp64"][:, :, 0, :], out["mixed"][:, :, 0, :]
    assert np.abs(rho_m - rho_f).sum() / np.abs(rho_f).sum() <= 1e-7


def test_kh_512_reruns_identical_and_mixed_tracks_fp64():
    n, nsteps = 512, 2
    res = {}
    for precision in ("fp64", "mixed"):
        runs = []
        for _ in range(2):
            with Solver(n, n, n, precision=precision) as s:
                s.init_kh(seed=1)
                s.step(nsteps)
                r = s.sync()
                assert r.step == nsteps and r.status == 0
                runs.append((r.dt, r.chg, r.time, tuple(s.diag())))
        assert runs[0] == runs[1], precision
        res[precision] = runs[0]
    f, m = res["fp64"], res["mixed"]
    assert abs(m[2] / f[2] - 1) <= 1e-5
    assert np.allclose(m[3], f[3], rtol=1e-5, atol=0)
