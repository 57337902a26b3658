"""The smallest grids the library accepts (2 cells on an axis).  A cell's ghost images then go to
both ends of the axis at once, every tile is partial, and the tensor-map box is larger than the
array.  Checked against the oracle after 5 steps for every boundary kind: the separately rounded
FP64 step bit for bit, the FMA-contracted one within 1e-11, the mixed form within 1e-4."""
import numpy as np
import pytest

import oracle as O
from mhdturbulence_gb300 import Solver, ic

pytestmark = pytest.mark.gpu
GAM = 5.0 / 3.0
P, R, F = ic.BC_PERIODIC, ic.BC_REFLECTION, ic.BC_OUTFLOW
SHAPES = [(2, 2, 2), (2, 3, 4), (3, 2, 2), (4, 3, 2), (5, 2, 3)]
BCS = [ic.KH_BC, (F,) * 6, (R,) * 6, (P, P, F, R, R, F)]


def rel_linf(a, b, floor=1e-3):
    err = 0.0
    for m in range(b.shape[2]):
        scale = max(np.abs(b[:, :, m, :]).max(), floor)
        err = max(err, np.abs(a[:, :, m, :] - b[:, :, m, :]).max() / scale)
    return err


@pytest.mark.parametrize("bc", BCS, ids=["kh", "outflow", "reflect", "mixed_bc"])
@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
def test_tiny_grids_vs_oracle(shape, bc):
    nx, ny, nz = shape
    nsteps = 5
    U0 = ic.prim_to_cons(ic.kh_prim(nx, ny, nz, seed=2), GAM)
    orc = O.Oracle(nx, ny, nz, *ic.grid(nx, ny, nz, ic.KH_DOMAIN), gam=GAM, bc=bc, spacing_quirk=False)
    Uo, Po = U0.copy(), ic.empty_field(nx, ny, nz, 12)
    orc.update_prim(Uo, Po)
    orc.run(Uo, Po, nsteps)
    ref = ic.interior(Uo)
    for precision, tol in (("fp64_exact", 0.0), ("fp64", 1e-11), ("mixed", 1e-4)):
        with Solver(nx, ny, nz, bc=bc, precision=precision) as s:
            s.upload_cons(U0)
            s.step(nsteps)
            r = s.sync()
            assert r.status == 0 and r.step == nsteps
            e = rel_linf(ic.interior(s.download_cons()), ref)
            assert e <= tol, (precision, e)
