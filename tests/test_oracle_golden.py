"""The oracle (oracle/mhd_oracle.c) against the golden vectors produced by the reference's own
src_cpp_kokkos_host stages: bit-for-bit equality of dt, c_h, P and U after 1 and N steps,
including the ghost layers for the case stored in full."""
import numpy as np
import pytest

import oracle as O
from golden_cases import cases
from mhdturbulence_gb300 import ic

CASES = cases()


@pytest.mark.parametrize("case", CASES, ids=[c.name for c in CASES])
def test_oracle_matches_reference_bitwise(case):
    orc = O.Oracle(case.nx, case.ny, case.nz, *case.axes(), gam=case.gam, bc=case.bc, spacing_quirk=True)
    U = case.U0()
    P = ic.empty_field(case.nx, case.ny, case.nz, 12)
    orc.update_prim(U, P)
    assert np.array_equal(case.view(P), case.z["P0"])
    _, dts, chgs = orc.run(U, P, 1)
    assert dts[0] == case.z["dts"][0] and chgs[0] == case.z["chgs"][0]
    assert np.array_equal(case.view(P), case.z["P1"])
    assert np.array_equal(case.view(U), case.z["U1"])
    _, dts, chgs = orc.run(U, P, case.nsteps - 1)
    assert np.array_equal(dts, case.z["dts"][1:]) and np.array_equal(chgs, case.z["chgs"][1:])
    assert np.array_equal(case.view(P), case.z["PN"])
    assert np.array_equal(case.view(U), case.z["UN"])


def test_oracle_stage_fluxes_match_reference():
    case = next(c for c in CASES if c.full)
    orc = O.Oracle(case.nx, case.ny, case.nz, *case.axes(), gam=case.gam, bc=case.bc, spacing_quirk=True)
    U = case.U0()
    P = ic.empty_field(case.nx, case.ny, case.nz, 12)
    orc.update_prim(U, P)
    orc.control_timestep(P)
    orc.set_boundary(P)
    chg = orc.evaluate_ch(P)
    assert chg == case.z["chgs"][0]
    for d in (1, 2, 3):
        F = orc.flux(d, P, chg)
        assert np.array_equal(F, case.z["F1"][d - 1]), f"flux dir {d}"


def test_oracle_thread_count_invariance():
    case = CASES[0]
    res = []
    for nt in (1, 3):
        O.set_threads(nt)
        orc = O.Oracle(case.nx, case.ny, case.nz, *case.axes(), gam=case.gam, bc=case.bc)
        U = case.U0()
        P = ic.empty_field(case.nx, case.ny, case.nz, 12)
        orc.update_prim(U, P)
        orc.run(U, P, 3)
        res.append(U.copy())
    O.set_threads(0)
    assert np.array_equal(res[0], res[1])
