"""Ensembles of independent grids advanced together (the batched form of the solver step).

Each member is a full grid with its own size, boundaries, gamma and state; every ensemble step is
one persistent launch of the fused kernel over the work items of all members (each member moving
by its own dt), captured in CUDA graphs.  Members are Solver objects borrowed from the ensemble.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import ic
from ._lib import Config, MhdgbError, Report, lib
from .solver import Solver, make_config

SIZES = (32, 48, 64, 96, 128)


def kh_ensemble_specs(n=64, seed=2026, sizes=SIZES):
    """Seeded uneven Kelvin-Helmholtz ensemble: grid extents drawn per axis from `sizes` (at most
    128^3 cells each), shear Mach number M ~ U[0.3, 1.5] (v_x = M c_s tanh(y/0.05) with
    c_s = sqrt(gamma p/rho) of the rho = p = 1 background), B_x ~ U[0, 0.3], and a noise seed each."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        nx, ny, nz = (int(rng.choice(sizes)) for _ in range(3))
        specs.append({"nx": nx, "ny": ny, "nz": nz, "mach": float(rng.uniform(0.3, 1.5)),
                      "bx": float(rng.uniform(0.0, 0.3)), "seed": int(rng.integers(1, 2 ** 31))})
    return specs


class Ensemble:
    def __init__(self, specs, precision="mixed", device=0, gam=5.0 / 3.0, cfl=0.05):
        self._L = lib()
        cfgs = (Config * len(specs))()
        for i, sp in enumerate(specs):
            cfgs[i] = make_config(sp["nx"], sp["ny"], sp["nz"], sp.get("domain", ic.KH_DOMAIN),
                                  sp.get("bc", ic.KH_BC), gam, cfl, precision, False, device)
        e = C.c_void_p()
        rc = self._L.mhdgb_ensemble_create(len(specs), cfgs, C.byref(e))
        if rc != 0:
            raise MhdgbError(rc, "mhdgb_ensemble_create failed")
        self._e = e
        self.specs = list(specs)
        self.precision = precision
        self.gam = gam
        self.members = []
        for i, sp in enumerate(specs):
            h = C.c_void_p()
            self._ck(self._L.mhdgb_ensemble_member(e, i, C.byref(h)), "member")
            self.members.append(Solver(sp["nx"], sp["ny"], sp["nz"], precision=precision, device=device,
                                       gam=gam, cfl=cfl, domain=sp.get("domain", ic.KH_DOMAIN),
                                       bc=sp.get("bc", ic.KH_BC), _borrow=h))
            if sp.get("riemann", "hlld") != "hlld":
                self.members[-1].set_riemann(sp["riemann"])

    def _ck(self, rc, what):
        if rc != 0:
            msg = self._L.mhdgb_ensemble_last_error(self._e)
            raise MhdgbError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "_e", None):
            for m in self.members:
                m._h = None
            self._L.mhdgb_ensemble_destroy(self._e)
            self._e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.members)

    @property
    def cells(self) -> int:
        return int(self._L.mhdgb_ensemble_cells(self._e))

    def init_kh(self, width=0.05, amp=1e-2, sig=0.2, noise=1e-4):
        """Each member's KH state from its spec (see kh_ensemble_specs)."""
        cs = np.sqrt(self.gam)
        for m, sp in zip(self.members, self.specs):
            m.init_kh(seed=sp["seed"], vshear=sp["mach"] * cs, width=width, bx=sp["bx"], amp=amp, sig=sig,
                      noise=noise)

    def prepare(self):
        self._ck(self._L.mhdgb_ensemble_prepare(self._e), "prepare")

    def step(self, n=1):
        self._ck(self._L.mhdgb_ensemble_step(self._e, n), "step")

    def sync(self):
        reps = (Report * len(self.members))()
        self._ck(self._L.mhdgb_ensemble_sync(self._e, reps), "sync")
        return list(reps)

    def set_stop(self, tmax=1e300, max_steps=-1):
        self._ck(self._L.mhdgb_ensemble_set_stop(self._e, tmax, max_steps), "set_stop")

    def time_steps(self, n) -> float:
        ms = C.c_double()
        self._ck(self._L.mhdgb_ensemble_time_steps(self._e, n, C.byref(ms)), "time_steps")
        return ms.value

    def select_variant(self, idx):
        self._ck(self._L.mhdgb_ensemble_select_variant(self._e, idx), "select_variant")

    @property
    def variant(self) -> int:
        return int(self._L.mhdgb_ensemble_variant(self._e))

    @property
    def variant_name(self) -> str:
        """Kernel form and tile shape every member runs."""
        return self.members[0].variant_name(-1)

    def autotune(self, steps=2) -> int:
        best = C.c_int()
        self._ck(self._L.mhdgb_ensemble_autotune(self._e, steps, C.byref(best)), "autotune")
        return best.value
