"""Block decomposition of one grid: the topology (the reference's MPI_Cart_create split,
src_cpp_kokkos_host/mpi_config.cpp:61-69) and the in-process domain of libmhdgb.so.

A domain cuts the grid into ntiles[0] x ntiles[1] x ntiles[2] blocks.  Each block is an ordinary
handle whose faces shared with another block have the kind BC_EXCHANGE; after every step the
halos of those faces are copied on the device(s) from the neighbouring blocks and dt / c_h are
reduced over all blocks (boundary.cpp:222-318 and mpi_config.cpp:83-99 in the reference).  Blocks
take their cell faces from the whole grid, so a decomposed run equals the single-grid run bit for
bit.  The multi-process form of the same split is mhdturbulence_gb300.distributed.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import ic
from ._lib import BC_EXCHANGE, Config, MhdgbError, Report, lib
from .solver import Solver, make_config

FACES = ("x-in", "x-out", "y-in", "y-out", "z-in", "z-out")


def cart_coords(rank: int, ntiles) -> tuple[int, int, int]:
    """Coordinates of a rank in the row-major order of MPI_Cart_create (last axis fastest)."""
    n0, n1, n2 = ntiles
    return rank // (n1 * n2), (rank // n2) % n1, rank % n2


def cart_rank(coords, ntiles) -> int:
    return (coords[0] * ntiles[1] + coords[1]) * ntiles[2] + coords[2]


def split_axis(n: int, nt: int, c: int) -> tuple[int, int]:
    """(first cell, cell count) of block c of nt along an axis of n cells; the first n % nt blocks
    take one cell more."""
    base, rem = divmod(n, nt)
    return c * base + min(c, rem), base + (1 if c < rem else 0)


def block_bc(bc, ntiles, coords) -> tuple[int, ...]:
    """Boundary kinds of a block: a face on the whole grid's boundary keeps its kind unless it wraps
    around to another block (periodic with more than one block along the axis); inner faces are
    exchanged."""
    out = []
    for f in range(6):
        a, side = divmod(f, 2)
        edge = coords[a] == (ntiles[a] - 1 if side else 0)
        out.append(bc[f] if edge and not (bc[f] == ic.BC_PERIODIC and ntiles[a] > 1) else BC_EXCHANGE)
    return tuple(out)


def neighbour(coords, face: int, ntiles) -> tuple[int, int, int]:
    """Coordinates of the block across `face` (wrapping around, as a periodic Cartesian topology)."""
    a, side = divmod(face, 2)
    c = list(coords)
    c[a] = (c[a] + (1 if side else -1)) % ntiles[a]
    return tuple(c)


def face_box(ext, face: int, ghost: bool):
    """Slices (k, j, i) of a block's array of extents ext = (nx, ny, nz) holding face `face`'s 2
    interior layers (ghost False) or the 2 ghost layers beyond it, over the interior transverse
    extent; ngh = 2."""
    a, side = divmod(face, 2)
    lo = [2, 2, 2]
    n = list(ext)
    lo[a] = (2 + n[a] if side else 0) if ghost else (2 + n[a] - 2 if side else 2)
    n[a] = 2
    return slice(lo[2], lo[2] + n[2]), slice(lo[1], lo[1] + n[1]), slice(lo[0], lo[0] + n[0])


class Domain:
    """One grid in blocks inside this process (mhdgb_domain_*).  groups / devices: the blocks run in
    len(devices) groups, block b in group b % len(devices) on devices[b % len(devices)]; None: one
    group on `device`."""

    def __init__(self, nx, ny, nz, ntiles, domain=ic.KH_DOMAIN, bc=ic.KH_BC, gam=5.0 / 3.0, cfl=0.05,
                 precision="fp64", device=0, devices=None):
        self._L = lib()
        cfg = make_config(nx, ny, nz, domain, bc, gam, cfl, precision, False, device)
        nt = (C.c_int * 3)(*ntiles)
        ndev = 0 if devices is None else len(devices)
        devs = None if devices is None else (C.c_int * ndev)(*devices)
        d = C.c_void_p()
        rc = self._L.mhdgb_domain_create(C.byref(cfg), nt, ndev, devs, C.byref(d))
        if rc != 0:
            msg = self._L.mhdgb_domain_last_error(d) if d else b""
            raise MhdgbError(rc, f"mhdgb_domain_create failed {msg.decode() if msg else ''}")
        self._d = d
        self.nx, self.ny, self.nz = nx, ny, nz
        self.ntiles = tuple(ntiles)
        self.precision = precision
        self.blocks = []
        for b in range(self._L.mhdgb_domain_blocks(d)):
            h, off, ext = C.c_void_p(), (C.c_int * 3)(), (C.c_int * 3)()
            self._ck(self._L.mhdgb_domain_block(d, b, C.byref(h), off, ext), "block")
            coords = cart_coords(b, self.ntiles)
            s = Solver(*ext, domain=domain, bc=block_bc(bc, self.ntiles, coords), gam=gam, cfl=cfl,
                       precision=precision, device=device, _borrow=h)
            s.offset = tuple(off)
            self.blocks.append(s)

    def _ck(self, rc, what):
        if rc != 0:
            msg = self._L.mhdgb_domain_last_error(self._d)
            raise MhdgbError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "_d", None):
            for s in self.blocks:
                s._h = None
            self._L.mhdgb_domain_destroy(self._d)
            self._d = None

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
        return np.zeros((self.nz + 5, self.ny + 5, nv, self.nx + 5), dtype=np.float64)

    def upload_cons(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        self._ck(self._L.mhdgb_domain_upload_cons(self._d, U.ctypes.data_as(C.POINTER(C.c_double))), "upload_cons")

    def download_cons(self):
        U = self.field(10)
        self._ck(self._L.mhdgb_domain_download_cons(self._d, U.ctypes.data_as(C.POINTER(C.c_double))),
                 "download_cons")
        return U

    def init_kh(self, seed=1, vshear=0.5, width=0.05, bx=0.1, amp=1e-2, sig=0.2, noise=1e-4):
        self._ck(self._L.mhdgb_domain_init_kh(self._d, seed, vshear, width, bx, amp, sig, noise), "init_kh")

    def prepare(self):
        self._ck(self._L.mhdgb_domain_prepare(self._d), "prepare")

    def step(self, n=1):
        self._ck(self._L.mhdgb_domain_step(self._d, n), "step")

    def sync(self) -> Report:
        r = Report()
        self._ck(self._L.mhdgb_domain_sync(self._d, C.byref(r)), "sync")
        return r

    def set_stop(self, tmax=1e300, max_steps=-1):
        self._ck(self._L.mhdgb_domain_set_stop(self._d, tmax, max_steps), "set_stop")

    def time_steps(self, n) -> float:
        ms = C.c_double()
        self._ck(self._L.mhdgb_domain_time_steps(self._d, n, C.byref(ms)), "time_steps")
        return ms.value

    def diag(self):
        out = np.zeros(3)
        self._ck(self._L.mhdgb_domain_diag(self._d, out.ctypes.data_as(C.POINTER(C.c_double))), "diag")
        return out


__all__ = ["Domain", "cart_coords", "cart_rank", "split_axis", "block_bc", "neighbour", "face_box", "FACES",
           "Config"]
