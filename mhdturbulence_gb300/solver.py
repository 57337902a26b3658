"""Python host mirror of the reference's stage interface, over the C ABI of libmhdgb.so.

The method names follow the reference's hydflux_mod / boundary_mod functions
(src_cpp_kokkos_host/mhd.hpp:277-287, boundary.hpp:139-144); arrays are numpy float64 in the
reference FieldArray layout, shape (ktot, jtot, nv, itot) (see ic.py).  Errors raise MhdgbError.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import ic
from ._lib import PRECISIONS, RIEMANN, Config, MhdgbError, Report, lib


def make_config(nx, ny, nz, domain=ic.KH_DOMAIN, bc=ic.KH_BC, gam=5.0 / 3.0, cfl=0.05, precision="fp64",
                spacing_quirk=False, device=0) -> Config:
    cfg = Config()
    lib().mhdgb_config_default(C.byref(cfg))
    cfg.nx, cfg.ny, cfg.nz = nx, ny, nz
    (cfg.x1min, cfg.x1max), (cfg.x2min, cfg.x2max), (cfg.x3min, cfg.x3max) = domain
    cfg.bc = (C.c_int * 6)(*bc)
    cfg.gam, cfg.cfl = gam, cfl
    cfg.precision = PRECISIONS[precision]
    cfg.spacing_quirk = 1 if spacing_quirk else 0
    cfg.device = device
    return cfg


def _dptr(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise ValueError("arrays must be C-contiguous float64")
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Solver:
    """One grid on one GPU.

    precision: "fp64" (FMA-contracted FP64), "fp64_exact" (separately rounded, the reference's
    arithmetic bit for bit) or "mixed" (FP32 reconstruction/Riemann solve, FP64 state, update,
    pressure recovery and reductions).  spacing_quirk reproduces mhd.cpp:1435-1436 (y/z spacing
    taken at index i in UpdateConservU).  riemann: "hlld" (the C++ path's), "hlle" or "hllc" (the
    Fortran variant's alternatives)."""

    def __init__(self, nx, ny, nz, domain=ic.KH_DOMAIN, bc=ic.KH_BC, gam=5.0 / 3.0, cfl=0.05,
                 precision="fp64", spacing_quirk=False, device=0, riemann="hlld", _borrow=None):
        self._L = lib()
        self._owned = _borrow is None
        cfg = make_config(nx, ny, nz, domain, bc, gam, cfl, precision, spacing_quirk, device)
        if _borrow is not None:
            self._h = _borrow
            self._setup(nx, ny, nz, precision, cfg)
            return
        h = C.c_void_p()
        rc = self._L.mhdgb_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise MhdgbError(rc, "mhdgb_create failed")
        self._h = h
        self._setup(nx, ny, nz, precision, cfg)
        if riemann != "hlld":
            self.set_riemann(riemann)

    def set_riemann(self, name):
        self._ck(self._L.mhdgb_set_riemann(self._h, RIEMANN[name]), "set_riemann")

    @property
    def riemann(self) -> str:
        code = self._L.mhdgb_get_riemann(self._h)
        return {v: k for k, v in RIEMANN.items()}[code]

    def _setup(self, nx, ny, nz, precision, cfg):
        h = self._h
        self.nx, self.ny, self.nz = nx, ny, nz
        self.precision = precision
        self.cfg = cfg
        it, jt, kt = C.c_int(), C.c_int(), C.c_int()
        self._L.mhdgb_extents(h, C.byref(it), C.byref(jt), C.byref(kt))
        self.itot, self.jtot, self.ktot = it.value, jt.value, kt.value

    # -- plumbing --
    def _ck(self, rc, what):
        if rc != 0:
            msg = self._L.mhdgb_last_error(self._h)
            raise MhdgbError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                self._L.mhdgb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def field(self, nv):
        return np.zeros((self.ktot, self.jtot, nv, self.itot), dtype=np.float64)

    @property
    def device_bytes(self) -> int:
        return int(self._L.mhdgb_device_bytes(self._h))

    # -- grid (GridArray) --
    def grid(self):
        a = [np.zeros(n) for n in (self.itot, self.jtot, self.ktot)]
        self._ck(self._L.mhdgb_get_grid(self._h, *(_dptr(x) for x in a)), "get_grid")
        return tuple(a)

    def set_grid(self, x1a, x2a, x3a):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (x1a, x2a, x3a)]
        self._ck(self._L.mhdgb_set_grid(self._h, *(_dptr(x) for x in a)), "set_grid")

    # -- transfers --
    def upload_cons(self, U):
        self._ck(self._L.mhdgb_upload_cons(self._h, _dptr(np.ascontiguousarray(U))), "upload_cons")

    def upload_prim(self, P):
        self._ck(self._L.mhdgb_upload_prim(self._h, _dptr(np.ascontiguousarray(P))), "upload_prim")

    def download_cons(self):
        U = self.field(10)
        self._ck(self._L.mhdgb_download_cons(self._h, _dptr(U)), "download_cons")
        return U

    def download_prim(self):
        P = self.field(12)
        self._ck(self._L.mhdgb_download_prim(self._h, _dptr(P)), "download_prim")
        return P

    def download_flux(self, d):
        F = self.field(10)
        self._ck(self._L.mhdgb_download_flux(self._h, d, _dptr(F)), "download_flux")
        return F

    # -- stage entry points (reference names) --
    def ControlTimestep(self) -> float:
        dt = C.c_double()
        self._ck(self._L.mhdgb_control_timestep(self._h, C.byref(dt)), "ControlTimestep")
        return dt.value

    def SetBoundaryCondition(self):
        self._ck(self._L.mhdgb_set_boundary(self._h), "SetBoundaryCondition")

    def EvaluateCh(self) -> float:
        ch = C.c_double()
        self._ck(self._L.mhdgb_evaluate_ch(self._h, C.byref(ch)), "EvaluateCh")
        return ch.value

    def GetNumericalFluxD(self, d: int):
        self._ck(self._L.mhdgb_flux(self._h, d), f"GetNumericalFluxD({d})")

    def UpdateConservU(self):
        self._ck(self._L.mhdgb_update_conserv(self._h), "UpdateConservU")

    def DampPsi(self):
        self._ck(self._L.mhdgb_damp_psi(self._h), "DampPsi")

    def UpdatePrimitvP(self):
        self._ck(self._L.mhdgb_update_prim(self._h), "UpdatePrimitvP")

    def set_dt(self, dt):
        self._ck(self._L.mhdgb_set_dt(self._h, dt), "set_dt")

    def set_chg(self, chg):
        self._ck(self._L.mhdgb_set_chg(self._h, chg), "set_chg")

    def stage_step(self):
        """One step through the stage entry points in the order of main.cpp:229-257."""
        dt = self.ControlTimestep()
        self.SetBoundaryCondition()
        chg = self.EvaluateCh()
        for d in (1, 2, 3):
            self.GetNumericalFluxD(d)
        self.UpdateConservU()
        self.DampPsi()
        self.UpdatePrimitvP()
        return dt, chg

    # -- fused step --
    def prepare(self):
        self._ck(self._L.mhdgb_prepare(self._h), "prepare")

    def step(self, n=1):
        self._ck(self._L.mhdgb_step(self._h, n), "step")

    def sync(self) -> Report:
        r = Report()
        self._ck(self._L.mhdgb_sync(self._h, C.byref(r)), "sync")
        return r

    def set_stop(self, tmax=1e300, max_steps=-1):
        self._ck(self._L.mhdgb_set_stop(self._h, tmax, max_steps), "set_stop")

    def run_until(self, tmax, max_steps=-1) -> Report:
        r = Report()
        self._ck(self._L.mhdgb_run_until(self._h, tmax, max_steps, C.byref(r)), "run_until")
        return r

    def reset_clock(self):
        self._ck(self._L.mhdgb_reset_clock(self._h), "reset_clock")

    def step_host(self, U_in, U_out, n=1):
        dt, ch = C.c_double(), C.c_double()
        self._ck(self._L.mhdgb_step_host(self._h, _dptr(U_in), _dptr(U_out), n, C.byref(dt), C.byref(ch)),
                 "step_host")
        return dt.value, ch.value

    def time_steps(self, n) -> float:
        """Device time (ms) of n fused steps, CUDA events on the launching stream."""
        ms = C.c_double()
        self._ck(self._L.mhdgb_time_steps(self._h, n, C.byref(ms)), "time_steps")
        return ms.value

    def variants(self):
        """[(tx, ty, threads, current)] of the compiled fused-kernel tile shapes."""
        out = []
        for v in range(self._L.mhdgb_variant_count(self._h)):
            tx, ty, nt, cur = C.c_int(), C.c_int(), C.c_int(), C.c_int()
            self._ck(self._L.mhdgb_variant_info(self._h, v, C.byref(tx), C.byref(ty), C.byref(nt), C.byref(cur)),
                     "variant_info")
            out.append((tx.value, ty.value, nt.value, bool(cur.value)))
        return out

    def variant_name(self, idx=-1) -> str:
        """Kernel form and tile shape of variant idx (-1: the kernel in use)."""
        name = self._L.mhdgb_variant_name(self._h, idx)
        if name is None:
            raise MhdgbError(-1, f"variant_name: no variant {idx}")
        return name.decode()

    def work_layout(self):
        """(tiles in x, tiles in y, z chunk lengths) of the fused step's work queue."""
        tx, ty, nc = C.c_int(), C.c_int(), C.c_int()
        self._ck(self._L.mhdgb_work_layout(self._h, C.byref(tx), C.byref(ty), C.byref(nc), None), "work_layout")
        ks = (C.c_int * (nc.value + 1))()
        self._ck(self._L.mhdgb_work_layout(self._h, None, None, None, ks), "work_layout")
        return tx.value, ty.value, [ks[i + 1] - ks[i] for i in range(nc.value)]

    def select_variant(self, idx):
        self._ck(self._L.mhdgb_select_variant(self._h, idx), "select_variant")

    def autotune(self, steps=4) -> int:
        best = C.c_int()
        self._ck(self._L.mhdgb_autotune(self._h, steps, C.byref(best)), "autotune")
        return best.value

    def diag(self):
        out = np.zeros(3)
        self._ck(self._L.mhdgb_diag(self._h, _dptr(out)), "diag")
        return out

    # -- snapshot output (Output, output.cpp:379-407) --
    def output_begin(self, root, index, time, dt, ascii=False):
        """Start writing snapshot `index` of the current state under root (bindata/, ascdata/);
        steps issued afterwards overlap the copy and the file writing."""
        self._ck(self._L.mhdgb_output_begin(self._h, os.fsencode(root), index, time, dt, 1 if ascii else 0),
                 "output_begin")

    def output_end(self):
        self._ck(self._L.mhdgb_output_end(self._h), "output_end")

    # -- checkpoint / restart --
    def checkpoint_save(self, path):
        self._ck(self._L.mhdgb_checkpoint_save(self._h, os.fsencode(path)), "checkpoint_save")

    def checkpoint_load(self, path):
        self._ck(self._L.mhdgb_checkpoint_load(self._h, os.fsencode(path)), "checkpoint_load")

    def output(self, root, index, time, dt, ascii=False):
        self._ck(self._L.mhdgb_output(self._h, os.fsencode(root), index, time, dt, 1 if ascii else 0), "output")

    # -- halo exchange of a block (faces shared with other blocks have the kind BC_EXCHANGE) --
    def halo_bytes(self, face) -> int:
        return int(self._L.mhdgb_halo_bytes(self._h, face))

    def halo_pack(self, face, buf_ptr):
        """Copy the 2 interior layers next to `face` into the device buffer at buf_ptr."""
        self._ck(self._L.mhdgb_halo_pack(self._h, face, buf_ptr), f"halo_pack({face})")

    def halo_unpack(self, face, buf_ptr):
        """Copy the device buffer at buf_ptr into the 2 ghost layers beyond `face`."""
        self._ck(self._L.mhdgb_halo_unpack(self._h, face, buf_ptr), f"halo_unpack({face})")

    def get_reduction(self):
        """(min cell CFL time, max signal speed) the next fused step will use (dt = cfl * the first)."""
        a, b = C.c_double(), C.c_double()
        self._ck(self._L.mhdgb_get_reduction(self._h, C.byref(a), C.byref(b)), "get_reduction")
        return a.value, b.value

    def set_reduction(self, dtmin, chmax):
        self._ck(self._L.mhdgb_set_reduction(self._h, dtmin, chmax), "set_reduction")

    def init_kh(self, seed=1, vshear=0.5, width=0.05, bx=0.1, amp=1e-2, sig=0.2, noise=1e-4):
        self._ck(self._L.mhdgb_init_kh(self._h, seed, vshear, width, bx, amp, sig, noise), "init_kh")

    def init_kh_block(self, whole, offset, seed=1, vshear=0.5, width=0.05, bx=0.1, amp=1e-2, sig=0.2, noise=1e-4):
        """The KH state of this block of a whole grid (cell counts `whole`, first cell `offset`)."""
        w, o = (C.c_int * 3)(*whole), (C.c_int * 3)(*offset)
        self._ck(self._L.mhdgb_init_kh_block(self._h, w, o, seed, vshear, width, bx, amp, sig, noise),
                 "init_kh_block")
