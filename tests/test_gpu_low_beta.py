"""The low-beta KH variant (B_x = 1, p = 0.1 on the KH layer, beta = 0.2) that stresses the FP64
pressure recovery of the mixed form.  The reference scheme amplifies any difference in this state
by about 3 % per step (the separately rounded FP64 form started from a state perturbed by 1e-15
drifts away geometrically and the state loses pressure positivity near step 280 in every form), so
the mixed form's distance from FP64 is FP32 rounding amplified by the scheme: it must stay at the
level that amplification predicts, density L1 <= 1e-5 over the first 140 steps at 128^3 (measured
4.5e-6), and the FMA-contracted FP64 form must stay within 1e-12 of the separately rounded one."""
import numpy as np
import pytest

from mhdturbulence_gb300 import Solver, ic

pytestmark = pytest.mark.gpu
GAM = 5.0 / 3.0


def _rho_after(prec, U0, n, marks):
    out = []
    with Solver(n, n, n, precision=prec) as s:
        s.upload_cons(U0)
        done = 0
        for m in marks:
            s.step(m - done)
            done = m
            r = s.sync()
            assert r.status == 0
            out.append(ic.interior(s.download_cons())[:, :, 0, :].copy())
    return out


def test_low_beta_mixed_and_fma_track_separately_rounded_fp64():
    n, marks = 128, (20, 140)
    U0 = ic.prim_to_cons(ic.kh_prim(n, n, n, seed=1, bx=1.0, p=0.1), GAM)
    ref = _rho_after("fp64_exact", U0, n, marks)
    fma = _rho_after("fp64", U0, n, marks)
    mix = _rho_after("mixed", U0, n, marks)

    def l1(a, b):
        return float(np.abs(a - b).sum() / np.abs(b).sum())

    for a, b in zip(fma, ref):
        assert l1(a, b) <= 1e-12
    assert l1(mix[0], ref[0]) <= 1e-6       # 20 steps: 1.1e-7 measured
    assert l1(mix[1], ref[1]) <= 1e-5       # 140 steps: 4.5e-6 measured
