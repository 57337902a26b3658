"""Operation counts of the solver step (oracle/flopcount.cpp).  The restatement compiled with an
operation-counting double must run the same arithmetic as the plain oracle: the same state, bit
for bit, after several steps.  Its per-cell counts are then those of the reference's algorithm,
with the face fluxes carrying most of the work."""
import numpy as np

import oracle as O
from mhdturbulence_gb300 import ic

GAM = 5.0 / 3.0


def test_counted_restatement_matches_plain_oracle_and_counts_the_step():
    nx, ny, nz, nsteps = 20, 24, 16, 3
    U0 = ic.prim_to_cons(ic.kh_prim(nx, ny, nz, seed=1), GAM)
    counts, U = O.count_ops(U0, nx, ny, nz, ic.KH_DOMAIN, ic.KH_BC, gam=GAM, nsteps=nsteps)
    orc = O.Oracle(nx, ny, nz, *ic.grid(nx, ny, nz, ic.KH_DOMAIN), gam=GAM, bc=ic.KH_BC, spacing_quirk=False)
    Uo, Po = U0.copy(), ic.empty_field(nx, ny, nz, 12)
    orc.update_prim(Uo, Po)
    orc.run(Uo, Po, nsteps)
    assert np.array_equal(U, Uo)

    assert counts["cells"] == nx * ny * nz and counts["steps"] == nsteps
    step = counts["step1"]
    assert step["div"] > 0 and step["sqrt"] > 0
    assert step["flops"] == step["add"] + step["mul"] + step["div"] + step["sqrt"]
    stages = counts["stages"]
    assert abs(sum(v["flops"] for v in stages.values()) - step["flops"]) <= 1e-6 * step["flops"]
    assert stages["SetBoundaryCondition"]["flops"] == 0.0  # copies only
    flux = sum(stages[f"GetNumericalFlux{d}"]["flops"] for d in (1, 2, 3))
    assert flux >= 0.8 * step["flops"]
