"""ctypes binding of the oracle (oracle/mhd_oracle.c).  TEST INFRASTRUCTURE ONLY.

Used by tests/ and __graft_entry__.smoke() as the reference the GPU results are compared with,
and by bench.py's CPU legs as the timed CPU baseline.  The shipped library never imports this module.
Arrays are numpy float64 in the reference FieldArray layout, shape (ktot, jtot, nv, itot).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


class OrcGrid(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("itot", C.c_int), ("jtot", C.c_int), ("ktot", C.c_int),
        ("gam", C.c_double), ("cfl", C.c_double),
        ("bc", C.c_int * 6), ("spacing_quirk", C.c_int),
        ("x1a", C.POINTER(C.c_double)), ("x2a", C.POINTER(C.c_double)), ("x3a", C.POINTER(C.c_double)),
        ("riemann", C.c_int),
    ]


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "mhd_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        gp = C.POINTER(OrcGrid)
        L.orc_flux.argtypes = [C.c_int, gp, dp, dp, C.c_double]
        L.orc_update_conserv.argtypes = [gp, dp, dp, dp, dp, C.c_double]
        L.orc_update_prim.argtypes = [gp, dp, dp]
        L.orc_control_timestep.argtypes = [gp, dp]
        L.orc_control_timestep.restype = C.c_double
        L.orc_evaluate_ch.argtypes = [gp, dp]
        L.orc_evaluate_ch.restype = C.c_double
        L.orc_damp_psi.argtypes = [gp, dp, C.c_double, C.c_double]
        L.orc_set_boundary.argtypes = [gp, dp]
        L.orc_step.argtypes = [gp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_run.argtypes = [gp, dp, dp, C.c_int, dp, dp]
        L.orc_run.restype = C.c_double
        L.orc_diag.argtypes = [gp, dp, dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """One grid configuration of the oracle; methods mirror the reference stage functions."""

    def __init__(self, nx, ny, nz, x1a, x2a, x3a, gam=5.0 / 3.0, cfl=0.05, bc=(1, 1, 2, 2, 1, 1),
                 spacing_quirk=True, riemann=0):
        self.axes = [np.ascontiguousarray(a, dtype=np.float64) for a in (x1a, x2a, x3a)]
        g = OrcGrid()
        g.nx, g.ny, g.nz = nx, ny, nz
        g.itot, g.jtot, g.ktot = nx + 5, ny + 5, nz + 5
        g.gam, g.cfl = gam, cfl
        g.bc = (C.c_int * 6)(*bc)
        g.spacing_quirk = 1 if spacing_quirk else 0
        g.riemann = riemann  # 0 HLLD, 1 HLLE, 2 HLLC
        g.x1a, g.x2a, g.x3a = (_ptr(a) for a in self.axes)
        self.g = g
        self.shape = (g.ktot, g.jtot, 0, g.itot)

    def field(self, nv):
        return np.zeros((self.g.ktot, self.g.jtot, nv, self.g.itot), dtype=np.float64)

    def flux(self, d, P, chg):
        F = self.field(10)
        lib().orc_flux(d, C.byref(self.g), _ptr(P), _ptr(F), chg)
        return F

    def update_conserv(self, Fx, Fy, Fz, U, dt):
        lib().orc_update_conserv(C.byref(self.g), _ptr(Fx), _ptr(Fy), _ptr(Fz), _ptr(U), dt)

    def update_prim(self, U, P):
        lib().orc_update_prim(C.byref(self.g), _ptr(U), _ptr(P))

    def control_timestep(self, P):
        return lib().orc_control_timestep(C.byref(self.g), _ptr(P))

    def evaluate_ch(self, P):
        return lib().orc_evaluate_ch(C.byref(self.g), _ptr(P))

    def damp_psi(self, U, dt, chg):
        lib().orc_damp_psi(C.byref(self.g), _ptr(U), dt, chg)

    def set_boundary(self, P):
        lib().orc_set_boundary(C.byref(self.g), _ptr(P))

    def run(self, U, P, nsteps):
        dts = np.zeros(max(nsteps, 1))
        chgs = np.zeros(max(nsteps, 1))
        t = lib().orc_run(C.byref(self.g), _ptr(U), _ptr(P), nsteps, _ptr(dts), _ptr(chgs))
        return t, dts[:nsteps], chgs[:nsteps]

    def diag(self, P):
        out = np.zeros(3)
        lib().orc_diag(C.byref(self.g), _ptr(P), _ptr(out))
        return out


def set_threads(n: int) -> None:
    lib().orc_set_threads(n)


def get_threads() -> int:
    return lib().orc_get_threads()


FLOPCOUNT_PATH = os.path.join(HERE, "_build", "flopcount")


def count_ops(U0, nx, ny, nz, domain, bc, gam=5.0 / 3.0, cfl=0.05, spacing_quirk=False, riemann=0, nsteps=1):
    """Operations per cell-update of the solver step, counted by running the restatement with an
    operation-counting double (oracle/flopcount.cpp): step 1 by stage, and the average over nsteps.
    Returns (counts, U after nsteps); the state equals the plain oracle's bit for bit."""
    import json
    import tempfile
    if not os.path.exists(FLOPCOUNT_PATH) or \
            os.path.getmtime(FLOPCOUNT_PATH) < os.path.getmtime(os.path.join(HERE, "mhd_oracle.c")) or \
            os.path.getmtime(FLOPCOUNT_PATH) < os.path.getmtime(os.path.join(HERE, "flopcount.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "flopcount"], check=True)
    U0 = np.ascontiguousarray(U0, dtype=np.float64)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "u0.bin"), os.path.join(d, "u1.bin")
        U0.tofile(fin)
        (x0, x1), (y0, y1), (z0, z1) = domain
        args = [FLOPCOUNT_PATH, nx, ny, nz, repr(float(gam)), repr(float(cfl)), *bc, int(bool(spacing_quirk)),
                riemann, repr(float(x0)), repr(float(x1)), repr(float(y0)), repr(float(y1)), repr(float(z0)),
                repr(float(z1)), fin, nsteps, fout]
        r = subprocess.run([str(a) for a in args], check=True, capture_output=True, text=True)
        U = np.fromfile(fout, dtype=np.float64).reshape(U0.shape)
    return json.loads(r.stdout), U
