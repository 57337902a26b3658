"""A block of a decomposed grid stepped by the oracle (test infrastructure): the block interface of
mhdturbulence_gb300.distributed, so the decomposition's host logic (topology, halo pairing and
order, reductions) runs among CPU ranks and can be compared bit for bit with the oracle's
single-grid run."""
import numpy as np
import torch

import oracle as O
from mhdturbulence_gb300 import ic
from mhdturbulence_gb300.distributed import block_geometry, sliced_axes
from mhdturbulence_gb300.domain import block_bc, face_box


class Report:
    def __init__(self, step, time, dt, chg):
        self.step, self.time, self.dt, self.chg, self.status = step, time, dt, chg, 0


class OracleBlock:
    transport = "cpu"
    halo_dtype = torch.float64

    def __init__(self, nx, ny, nz, ntiles, coords, domain=ic.KH_DOMAIN, bc=ic.KH_BC, gam=5.0 / 3.0, cfl=0.05):
        self.coords, self.ntiles = tuple(coords), tuple(ntiles)
        self.offset, self.extent = block_geometry(nx, ny, nz, ntiles, coords)
        self.bc = block_bc(bc, ntiles, coords)
        self.cfl = cfl
        axes = sliced_axes(nx, ny, nz, domain, self.offset, self.extent)
        self.orc = O.Oracle(*self.extent, *axes, gam=gam, cfl=cfl, bc=self.bc, spacing_quirk=False)
        # the same grid with CFL factor 1: control_timestep then returns the bare minimum
        self.orc_min = O.Oracle(*self.extent, *axes, gam=gam, cfl=1.0, bc=self.bc, spacing_quirk=False)
        self.P = self.orc.field(12)
        self.U = None
        self.nstep, self.time, self.last = 0, 0.0, (0.0, 0.0)

    def init_kh_from_whole(self, U_whole):
        o, e = self.offset, self.extent
        # a copy: a slice along k alone would be a view of the whole-grid array, which this block steps in place
        self.U = np.array(U_whole[o[2]:o[2] + e[2] + 5, o[1]:o[1] + e[1] + 5, :, o[0]:o[0] + e[0] + 5], copy=True)

    def _end_of_step(self):
        # P from U, ghosts of the faces that are not exchanged, the local reduction
        self.orc.update_prim(self.U, self.P)
        self.orc.set_boundary(self.P)
        self.pending = (self.orc_min.control_timestep(self.P), self.orc.evaluate_ch(self.P))

    def prepare(self):
        self._end_of_step()

    def step(self):
        dtmin, chg = self.pending
        dt = self.cfl * dtmin
        F = [self.orc.flux(d, self.P, chg) for d in (1, 2, 3)]
        self.orc.update_conserv(*F, self.U, dt)
        self.orc.damp_psi(self.U, dt, chg)
        self.time += dt
        self.nstep += 1
        self.last = (dt, chg)
        self._end_of_step()

    def pack(self, face):
        ks, js, is_ = face_box(self.extent, face, ghost=False)
        return torch.from_numpy(np.ascontiguousarray(self.P[ks, js, :, is_].transpose(2, 0, 1, 3)).reshape(-1))

    def unpack(self, face, t):
        ks, js, is_ = face_box(self.extent, face, ghost=True)
        box = self.P[ks, js, :, is_]
        self.P[ks, js, :, is_] = t.numpy().reshape(box.shape[2], box.shape[0], box.shape[1], box.shape[3]) \
            .transpose(1, 2, 0, 3)

    def get_reduction(self):
        return self.pending

    def set_reduction(self, dtmin, chmax):
        self.pending = (dtmin, chmax)

    def sync(self):
        return Report(self.nstep, self.time, *self.last)

    def download_cons(self):
        return self.U.copy()
