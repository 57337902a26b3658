"""Accuracy and throughput studies of the mixed and FP64 forms (GPU).

    python -m mhdturbulence_gb300.studies turbulence [--n 256 --steps 200]
    python -m mhdturbulence_gb300.studies kh_growth  [--n 128 --tmax 6]
    python -m mhdturbulence_gb300.studies ensemble   [--members 64 --steps 20]
    python -m mhdturbulence_gb300.studies low_beta   [--n 128 --steps 180]
    python -m mhdturbulence_gb300.studies all

Each prints one JSON object per study.
  turbulence: decaying turbulence (log-normal density, k^-2 velocity and vector-potential spectra,
    <B_x> = 0.2, beta ~ 10) on a periodic n^3 cube, `steps` steps in both forms; errors of the mixed
    form against FP64 (density L1/Linf, energy, div B) and conservation of mass and energy.
  kh_growth: the KH layer to tmax in both forms with sqrt(<v_y^2>) sampled along the way; growth
    rate Gamma fitted over the exponential phase 1 < t < 4 (the layer saturates near t = 4.5 at
    these resolutions); also the low-beta variant (B_x = 1, p = 0.1) over its stable window.
  ensemble: the seeded uneven 64-grid KH ensemble in both forms; aggregate Gcell-updates/s next to a
    single 512^3 grid and the per-grid error of the mixed form against FP64.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import ic
from ._lib import MhdgbError
from .ensemble import Ensemble, kh_ensemble_specs
from .solver import Solver

GAM = 5.0 / 3.0


def _divb_rms(P, axes):
    x1a, x2a, x3a = axes
    n3, n2, _, n1 = P.shape
    dx = np.diff(x1a)[2:2 + n1]
    dy = np.diff(x2a)[2:2 + n2]
    dz = np.diff(x3a)[2:2 + n3]
    bx, by, bz = P[:, :, ic.NBM1, :], P[:, :, ic.NBM2, :], P[:, :, ic.NBM3, :]
    d = (np.roll(bx, -1, 2) - np.roll(bx, 1, 2)) / (2 * dx[None, None, :]) \
        + (np.roll(by, -1, 1) - np.roll(by, 1, 1)) / (2 * dy[None, :, None]) \
        + (np.roll(bz, -1, 0) - np.roll(bz, 1, 0)) / (2 * dz[:, None, None])
    return float(np.sqrt(np.mean(d ** 2)))


def turbulence(n=256, steps=200, seed=7):
    U0 = ic.prim_to_cons(ic.turbulence_prim(n, seed=seed), GAM)
    out = {}
    for prec in ("fp64", "mixed"):
        with Solver(n, n, n, domain=ic.CUBE_DOMAIN, bc=ic.PERIODIC_BC, precision=prec) as s:
            s.upload_cons(U0)
            divb0 = _divb_rms(ic.interior(s.download_prim()), s.grid())
            s.autotune(steps=2)
            t0 = time.perf_counter()
            s.step(steps)
            r = s.sync()
            wall = time.perf_counter() - t0
            U = ic.interior(s.download_cons())
            P = ic.interior(s.download_prim())
            out[prec] = dict(r=r, U=U, P=P, divb0=divb0, divb=_divb_rms(P, s.grid()), wall=wall)
    d, m = out["fp64"], out["mixed"]
    U0i = ic.interior(U0)
    rho_d, rho_m = d["U"][:, :, 0, :], m["U"][:, :, 0, :]
    res = {
        "study": "turbulence", "n": n, "steps": steps, "time_fp64": d["r"].time, "time_mixed": m["r"].time,
        "rho_l1_rel": float(np.abs(rho_m - rho_d).sum() / np.abs(rho_d).sum()),
        "rho_linf_rel": float(np.abs(rho_m - rho_d).max() / np.abs(rho_d).max()),
        "energy_l1_rel": float(np.abs(m["U"][:, :, 4, :] - d["U"][:, :, 4, :]).sum() / np.abs(d["U"][:, :, 4, :]).sum()),
        "divB_rms_initial": d["divb0"], "divB_rms_fp64": d["divb"], "divB_rms_mixed": m["divb"],
        "mass_drift_fp64": float(abs(d["U"][:, :, 0, :].sum() / U0i[:, :, 0, :].sum() - 1)),
        "mass_drift_mixed": float(abs(m["U"][:, :, 0, :].sum() / U0i[:, :, 0, :].sum() - 1)),
        "energy_drift_fp64": float(abs(d["U"][:, :, 4, :].sum() / U0i[:, :, 4, :].sum() - 1)),
        "energy_drift_mixed": float(abs(m["U"][:, :, 4, :].sum() / U0i[:, :, 4, :].sum() - 1)),
        "wall_s_fp64": d["wall"], "wall_s_mixed": m["wall"],
    }
    return res


def _kh_series(n, prec, tmax, sample_every, bx, p, vshear, max_steps=-1):
    with Solver(n, n, n, precision=prec) as s:
        U0 = ic.prim_to_cons(ic.kh_prim(n, n, n, seed=1, bx=bx, p=p, vshear=vshear), GAM)
        s.upload_cons(U0)
        s.set_stop(tmax, max_steps)
        ts, vy = [0.0], [float(s.diag()[2])]
        t0 = time.perf_counter()
        while True:
            s.step(sample_every)
            r = s.sync()
            d = s.diag()
            ts.append(r.time)
            vy.append(float(d[2]))
            if r.done:
                break
        wall = time.perf_counter() - t0
        U = ic.interior(s.download_cons())
        P = ic.interior(s.download_prim())
    return np.array(ts), np.array(vy), r, wall, U, P


def _fit_growth(t, v, t0=1.0, t1=6.0):
    sel = (t >= t0) & (t <= t1) & (v > 0)
    if sel.sum() < 3:
        return None
    a, b = np.polyfit(t[sel], np.log(v[sel]), 1)
    return float(a)


def _first_bad_step(n, bx, p, limit, precision="fp64"):
    """First step at which the low-beta state has a non-finite or non-positive cell (the status
    word of that step's sync), or None if it survives `limit` steps; the reference scheme has no
    positivity fix."""
    with Solver(n, n, n, precision=precision) as s:
        s.upload_cons(ic.prim_to_cons(ic.kh_prim(n, n, n, seed=1, bx=bx, p=p), GAM))
        for k in range(1, limit + 1):
            s.step(1)
            try:
                s.sync()
            except MhdgbError:
                return k
    return None


def kh_growth(n=128, tmax=6.0, sample_every=200, low_beta_steps=None):
    """KH growth in both forms.  The low-beta variant (B_x = 1, p = 0.1) loses pressure positivity
    under the reference scheme within a few hundred steps (the oracle does too), in each form at its
    own step, so it is compared over the first 3/4 of the steps both forms survive, where the FP64
    pressure recovery matters most."""
    res = {"study": "kh_growth", "n": n, "tmax": tmax}
    bad = {prec: _first_bad_step(n, 1.0, 0.1, 400, prec) for prec in ("fp64", "mixed")}
    first = min((b for b in bad.values() if b), default=None)
    if low_beta_steps is None:
        low_beta_steps = max(1, (first - 1) * 3 // 4) if first else 100
    res["low_beta_first_failing_step_fp64"] = bad["fp64"]
    res["low_beta_first_failing_step_mixed"] = bad["mixed"]
    for name, bx, p, steps in (("kh", 0.1, 1.0, -1), ("low_beta", 1.0, 0.1, low_beta_steps)):
        runs = {}
        for prec in ("fp64", "mixed"):
            every = sample_every if steps < 0 else max(1, steps // 10)
            runs[prec] = _kh_series(n, prec, tmax, every, bx, p, 0.5, max_steps=steps)
        (td, vd, rd, wd, Ud, Pd), (tm, vm, rm, wm, Um, Pm) = runs["fp64"], runs["mixed"]
        vm_on_td = np.interp(td, tm, vm)
        out = {
            "bx": bx, "p": p, "steps_fp64": rd.step, "steps_mixed": rm.step, "t_end": float(td[-1]),
            "vy_rms_final_fp64": float(vd[-1]), "vy_rms_final_mixed": float(vm[-1]),
            "vy_series_max_rel_diff": float(np.max(np.abs(vm_on_td - vd) / np.maximum(np.abs(vd), 1e-30))),
            "rho_l1_rel_final": float(np.abs(Um[:, :, 0, :] - Ud[:, :, 0, :]).sum() / np.abs(Ud[:, :, 0, :]).sum()),
            "p_linf_rel_final": float(np.abs(Pm[:, :, 5, :] - Pd[:, :, 5, :]).max() / np.abs(Pd[:, :, 5, :]).max()),
            "p_l1_rel_final": float(np.abs(Pm[:, :, 5, :] - Pd[:, :, 5, :]).sum() / np.abs(Pd[:, :, 5, :]).sum()),
            "wall_s_fp64": wd, "wall_s_mixed": wm,
        }
        if steps < 0:
            gd, gm = _fit_growth(td, vd, 1.0, min(tmax, 4.0)), _fit_growth(tm, vm, 1.0, min(tmax, 4.0))
            out.update({"gamma_fit_window": [1.0, min(tmax, 4.0)], "gamma_fp64": gd, "gamma_mixed": gm,
                        "gamma_rel_diff": (abs(gm / gd - 1) if gd and gm else None),
                        "series_fp64": [[float(a), float(b)] for a, b in
                                        zip(td[::max(1, len(td) // 40)], vd[::max(1, len(td) // 40)])]})
        res[name] = out
    return res


def low_beta_sensitivity(n=128, steps=180, every=20, eps=1e-15, seed=11):
    """How the low-beta KH variant (B_x = 1, p = 0.1) amplifies perturbations.  Four runs from the
    same state: the separately rounded FP64 form (the reference's arithmetic), the FMA-contracted
    FP64 form, the mixed form, and the separately rounded form started from the state with each
    conserved value multiplied by (1 + eps * u), u uniform in [-1, 1] per cell (seeded).  Density L1
    distances between pairs every `every` steps show whether the mixed form's distance from FP64 is
    its own error or the scheme's amplification of any difference at the level of rounding."""
    U0 = ic.prim_to_cons(ic.kh_prim(n, n, n, seed=1, bx=1.0, p=0.1), GAM)
    rng = np.random.default_rng(seed)
    Up = U0 * (1.0 + eps * rng.uniform(-1.0, 1.0, size=U0.shape))
    runs = {"exact": ("fp64_exact", U0), "fma": ("fp64", U0), "mixed": ("mixed", U0), "perturbed": ("fp64_exact", Up)}
    rho = {name: [] for name in runs}
    marks = list(range(every, steps + 1, every))
    for name, (prec, U) in runs.items():
        with Solver(n, n, n, precision=prec) as s:
            s.upload_cons(U)
            done = 0
            for m in marks:
                s.step(m - done)
                done = m
                try:
                    s.sync()
                except MhdgbError:
                    rho[name].append(None)
                    break
                rho[name].append(ic.interior(s.download_cons())[:, :, 0, :].copy())

    def dist(a, b):
        return [None if x is None or y is None else float(np.abs(x - y).sum() / np.abs(y).sum())
                for x, y in zip(rho[a], rho[b])]
    res = {"study": "low_beta_sensitivity", "n": n, "bx": 1.0, "p": 0.1, "steps": marks, "eps": eps,
           "rho_l1_fma_vs_exact": dist("fma", "exact"), "rho_l1_mixed_vs_exact": dist("mixed", "exact"),
           "rho_l1_mixed_vs_fma": dist("mixed", "fma"), "rho_l1_perturbed_vs_exact": dist("perturbed", "exact")}
    pe = [v for v in res["rho_l1_perturbed_vs_exact"] if v]
    if len(pe) >= 2:  # growth of the planted difference per step
        res["perturbation_growth_per_step"] = float((pe[-1] / pe[0]) ** (1.0 / (marks[len(pe) - 1] - marks[0])))
    return res


def ensemble(members=64, steps=20, err_steps=50, big=512, seed=2026):
    specs = kh_ensemble_specs(members, seed=seed)
    res = {"study": "ensemble", "members": members, "cells": int(sum(s["nx"] * s["ny"] * s["nz"] for s in specs))}
    finals = {}
    for prec, k in (("mixed", steps), ("fp64", max(2, steps // 8))):
        with Ensemble(specs, precision=prec) as ens:
            ens.init_kh()
            best = ens.autotune(steps=2)
            ens.time_steps(3)
            ms = ens.time_steps(k)
            res[f"{prec}_gcells"] = ens.cells * k / (ms * 1e-3) / 1e9
            res[f"{prec}_tile_variant"] = best
        with Ensemble(specs, precision=prec) as ens:
            ens.init_kh()
            ens.step(err_steps)
            ens.sync()
            finals[prec] = [ic.interior(m.download_cons()) for m in ens.members]
        with Solver(big, big, big, precision=prec) as s:
            s.init_kh(seed=1)
            s.autotune(steps=2)
            s.time_steps(2)
            kk = 5 if prec == "mixed" else 2
            ms = s.time_steps(kk)
            res[f"{prec}_single_{big}_gcells"] = big ** 3 * kk / (ms * 1e-3) / 1e9
        res[f"{prec}_ratio_vs_single"] = res[f"{prec}_gcells"] / res[f"{prec}_single_{big}_gcells"]
    errs = []
    for a, b in zip(finals["mixed"], finals["fp64"]):
        errs.append(float(np.abs(a[:, :, 0, :] - b[:, :, 0, :]).sum() / np.abs(b[:, :, 0, :]).sum()))
    res["per_member_rho_l1_rel"] = {"steps": err_steps, "max": max(errs), "median": float(np.median(errs)),
                                    "min": min(errs)}
    return res


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["turbulence", "kh_growth", "ensemble", "low_beta", "all"])
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--tmax", type=float, default=6.0)
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--big", type=int, default=512)
    a = ap.parse_args(argv)
    todo = ["turbulence", "kh_growth", "ensemble"] if a.study == "all" else [a.study]
    for st in todo:
        if st == "turbulence":
            r = turbulence(n=a.n or 256, steps=a.steps or 200)
        elif st == "kh_growth":
            r = kh_growth(n=a.n or 128, tmax=a.tmax)
        elif st == "low_beta":
            r = low_beta_sensitivity(n=a.n or 128, steps=a.steps or 180)
        else:
            r = ensemble(members=a.members, steps=a.steps or 20, big=a.big)
        print(json.dumps(r), flush=True)


if __name__ == "__main__":
    sys.exit(main())
