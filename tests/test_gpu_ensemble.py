"""The batched ensemble form: every member of an ensemble advances exactly as the same grid run
alone (same precision and tile shape: the per-cell arithmetic is identical), with its own dt."""
import numpy as np
import pytest

from mhdturbulence_gb300 import Ensemble, Solver, ic, kh_ensemble_specs

pytestmark = pytest.mark.gpu


def _specs():
    specs = kh_ensemble_specs(5, seed=7, sizes=(16, 24, 32))
    # mixed boundaries and one periodic cube among the members
    specs[1]["bc"] = (ic.BC_OUTFLOW, ic.BC_REFLECTION, ic.BC_PERIODIC, ic.BC_PERIODIC, ic.BC_REFLECTION,
                      ic.BC_OUTFLOW)
    specs[3]["bc"] = ic.PERIODIC_BC
    specs[3]["domain"] = ic.CUBE_DOMAIN
    return specs


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ensemble_members_match_single_grid_runs(precision):
    specs = _specs()
    nsteps = 21
    with Ensemble(specs, precision=precision) as ens:
        ens.init_kh()
        U0 = [m.download_cons() for m in ens.members]
        ens.step(nsteps)
        reps = ens.sync()
        out = [m.download_cons() for m in ens.members]
        var = ens.variant
    dts = set()
    for sp, u0, u1, r in zip(specs, U0, out, reps):
        assert r.step == nsteps
        dts.add(r.dt)
        with Solver(sp["nx"], sp["ny"], sp["nz"], precision=precision, domain=sp.get("domain", ic.KH_DOMAIN),
                    bc=sp.get("bc", ic.KH_BC)) as s:
            s.select_variant(var)
            s.upload_cons(u0)
            s.step(nsteps)
            r1 = s.sync()
            assert np.array_equal(s.download_cons(), u1)
            assert r1.time == r.time
    assert len(dts) == len(specs)  # every member moved by its own dt


def test_ensemble_autotune_and_variants_agree():
    specs = _specs()
    results = []
    with Ensemble(specs, precision="mixed") as ens:
        ens.init_kh()
        U0 = [m.download_cons() for m in ens.members]
        best = ens.autotune(steps=2)
        assert ens.variant == best
        for m, u in zip(ens.members, U0):  # autotune restores every member
            assert np.array_equal(m.download_cons(), u)
        for v in range(len(ens.members[0].variants())):
            ens.select_variant(v)
            for m, u in zip(ens.members, U0):
                m.upload_cons(u)
                m.reset_clock()
                m.upload_cons(u)
            ens.step(5)
            ens.sync()
            results.append([m.download_cons() for m in ens.members])
    # mixed form: variants of one register budget agree bit for bit, the 1-CTA and 2-CTA builds
    # within 1e-9 relative (different FP32 multiply-add contraction)
    for r in results[1:]:
        for a, b in zip(r, results[0]):
            ai, bi = ic.interior(a), ic.interior(b)
            err = max(np.abs(ai[:, :, m, :] - bi[:, :, m, :]).max() / max(np.abs(bi[:, :, m, :]).max(), 1e-3)
                      for m in range(10))
            assert err <= 1e-9, err


def test_ensemble_stop_condition_per_member():
    specs = _specs()[:3]
    with Ensemble(specs, precision="fp64") as ens:
        ens.init_kh()
        ens.set_stop(tmax=1e300, max_steps=4)
        ens.members[1].set_stop(1e300, 2)
        ens.step(6)
        reps = ens.sync()
        assert [r.step for r in reps] == [4, 2, 4]
        assert all(r.done for r in reps)


def test_ensemble_members_exact_vs_oracle():
    """Each member of an uneven ensemble in the separately rounded FP64 form equals the oracle (the
    reference's stage arithmetic bit for bit) run on that member's grid: state, time and every
    step's dt and c_h."""
    import oracle as O

    specs = kh_ensemble_specs(4, seed=11, sizes=(12, 20, 28))
    specs[0]["bc"] = (ic.BC_REFLECTION, ic.BC_OUTFLOW, ic.BC_PERIODIC, ic.BC_PERIODIC, ic.BC_OUTFLOW,
                      ic.BC_REFLECTION)
    specs[2]["bc"] = ic.PERIODIC_BC
    specs[2]["domain"] = ic.CUBE_DOMAIN
    nsteps = 12
    with Ensemble(specs, precision="fp64_exact") as ens:
        ens.init_kh()
        U0 = [m.download_cons() for m in ens.members]
        got_dt = [[] for _ in specs]
        for _ in range(nsteps):
            ens.step(1)
            for q, r in enumerate(ens.sync()):
                got_dt[q].append((r.dt, r.chg))
        reps = ens.sync()
        out = [ic.interior(m.download_cons()) for m in ens.members]
    for q, (sp, u0) in enumerate(zip(specs, U0)):
        nx, ny, nz = sp["nx"], sp["ny"], sp["nz"]
        domain, bc = sp.get("domain", ic.KH_DOMAIN), sp.get("bc", ic.KH_BC)
        orc = O.Oracle(nx, ny, nz, *ic.grid(nx, ny, nz, domain), gam=5.0 / 3.0, bc=bc, spacing_quirk=False)
        U, P = u0.copy(), ic.empty_field(nx, ny, nz, 12)
        orc.update_prim(U, P)
        t, dts, chgs = orc.run(U, P, nsteps)
        assert np.array_equal(out[q], ic.interior(U)), q
        assert got_dt[q] == list(zip(dts.tolist(), chgs.tolist())), q
        assert reps[q].time == t, q


def test_new_grids_start_on_the_preferred_kernels():
    """Before any autotuning a grid or ensemble starts on the table entry marked as the fastest
    measured at the benchmark sizes: the two-phase 16x8/256 kernel in FP64 and the fused-slope
    16x8/256 kernel compiled for two CTAs per SM in the mixed form; HLLE/HLLC run on the run-time
    solver kernel."""
    want = {"fp64": "two-phase 16x8/256", "mixed": "fused-slope 16x8/256 x2", "fp64_exact": "two-phase 32x4/128"}
    for precision, name in want.items():
        with Solver(150, 150, 150, precision=precision) as s:
            assert s.variant_name() == name, precision
            s.set_riemann("hllc")
            assert s.variant_name().endswith("run-time solver"), precision
            s.set_riemann("hlld")
            assert s.variant_name() == name, precision
        with Ensemble(kh_ensemble_specs(3, seed=5, sizes=(16, 24)), precision=precision) as ens:
            assert ens.variant_name == name, precision


def test_work_queue_chunks_cover_the_grid():
    """The z chunks of the work queue cover every plane once, shrink towards the end of the queue
    where that balances the CTAs better, and do not change the results."""
    for n, precision in ((150, "fp64"), (150, "mixed"), (256, "mixed"), (40, "fp64")):
        with Solver(n, n, n, precision=precision) as s:
            ntx, nty, chunks = s.work_layout()
            assert sum(chunks) == n and min(chunks) >= 1 and len(chunks) <= 64, (n, precision, chunks)
            assert ntx * 16 >= n and nty * 8 >= n
    # same state with the grid's own chunking and with an ensemble's equal chunks
    specs = [{"nx": 48, "ny": 40, "nz": 45, "mach": 0.4, "bx": 0.1, "seed": 1}]
    with Ensemble(specs, precision="fp64") as ens, Solver(48, 40, 45, precision="fp64") as s:
        ens.init_kh()
        s.upload_cons(ens.members[0].download_cons())
        assert s.work_layout()[2] != ens.members[0].work_layout()[2]
        ens.step(9)
        s.step(9)
        ens.sync()
        s.sync()
        assert np.array_equal(ens.members[0].download_cons(), s.download_cons())
