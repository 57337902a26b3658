"""Loader for the golden vectors under tests/golden/ (made by tests/golden/make_golden.py from
the reference's own solver stages)."""
import glob
import os

import numpy as np

from mhdturbulence_gb300 import ic

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class Case:
    def __init__(self, path):
        z = np.load(path)
        self.name = os.path.splitext(os.path.basename(path))[0]
        self.nx, self.ny, self.nz, self.nsteps = (int(v) for v in z["meta"][:4])
        self.bc = tuple(int(b) for b in z["meta"][4:])
        self.domain = [tuple(r) for r in z["domain"]]
        self.gam = float(z["gam"][0])
        self.z = {k: z[k] for k in z.files}
        self.full = self.z["P1"].shape[0] == self.nz + 2 * ic.NGH + 1

    def axes(self):
        return ic.grid(self.nx, self.ny, self.nz, self.domain)

    def U0(self):
        U = ic.empty_field(self.nx, self.ny, self.nz, 10)
        ic.interior(U)[...] = self.z["U0"]
        return U

    def view(self, a):
        """The part of a full array that this case stores."""
        return a if self.full else ic.interior(a)


def cases():
    """The stage cases (every .npz but the output case output_*.npz)."""
    paths = sorted(glob.glob(os.path.join(HERE, "*.npz")))
    return [Case(p) for p in paths if not os.path.basename(p).startswith("output_")]
