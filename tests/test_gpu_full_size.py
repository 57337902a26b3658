"""The benchmark-size workloads.  KH on the 150^3 benchmark grid is checked against the oracle
directly (the oracle steps 150^3 in a fraction of a second on the host's cores).  Decaying
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


def test_turbulence_256_conserves_and_mixed_tracks_fp64():
    n, nsteps = 256, 10
    U0 = ic.prim_to_cons(ic.turbulence_prim(n, seed=4), GAM)
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
