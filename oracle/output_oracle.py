"""CPU restatement of the reference's snapshot output (test infrastructure: only the tests read it).

Follows src_cpp_kokkos_host/output.cpp for one rank:
  MPI_IO_Pack  (output.cpp:204-268)  interior primitives reordered to [var][z][y][x] FP64 with the
               variables d, v1, v2, v3, b1, b2, b3, bp, p, X1 (nden, nve1..3, nbm1..3, nbps, npre, nst);
               grids [2][n+1] per axis: cell centres x?b then faces x?a from index is (ngh) on;
  MPI_IO_Write (output.cpp:81-202)   bindata/unf%05d.dat text header, bindata/grid{1,2,3}D.bin,
               bindata/field%05d.bin (the single-rank subarray views cover whole files);
  WriteXDMF    (output.cpp:273-343)  bindata/field%05d.xmf;
  ASC_WRITE    (output.cpp:348-386)  ascdata/snap000-%05d.csv of the plane k = ks, %.6e formatting.
The reference's own output.cpp, run on the same inputs, produced tests/golden/output_7x5x4.npz, and
tests/test_output_golden.py checks this restatement against those files byte for byte.
"""
from __future__ import annotations

import os

import numpy as np

NGH = 2
# [var] order of field%05d.bin (output.cpp:247-260) as primitive indices, and the XDMF names
PACK_ORDER = (0, 1, 2, 3, 7, 8, 9, 10, 5, 11)
NAMES = ("d", "v1", "v2", "v3", "b1", "b2", "b3", "bp", "p", "X1")


def centres(xa: np.ndarray) -> np.ndarray:
    """x?b(i) = 0.5*(x?a(i+1) + x?a(i)) (GenerateGrid, main.cpp:42-44)."""
    return 0.5e0 * (xa[1:] + xa[:-1])


def pack(P: np.ndarray, nx: int, ny: int, nz: int) -> np.ndarray:
    """Fieldout of MPI_IO_Pack: P (ktot, jtot, 12, itot) -> (10, nz, ny, nx)."""
    inner = P[NGH:NGH + nz, NGH:NGH + ny, :, NGH:NGH + nx]
    return np.ascontiguousarray(np.stack([inner[:, :, n, :] for n in PACK_ORDER]))


def grid_block(xa: np.ndarray, n: int) -> np.ndarray:
    """grid?D.bin: [2][n+1] = (x?b, x?a) from index is = ngh."""
    return np.stack([centres(xa)[NGH:NGH + n + 1], xa[NGH:NGH + n + 1]])


def xdmf(nx: int, ny: int, nz: int, time: float, index: int) -> str:
    fdata = f"field{index:05d}.bin"
    out = ['<?xml version="1.0" ?>\n', '<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>\n', '<Xdmf Version="2.0">\n',
           "  <Domain>\n", '    <Grid Name="Grid" GridType="Uniform">\n', f'      <Time Value="{time:.16e}"/>\n',
           f'      <Topology TopologyType="3DRectMesh" Dimensions="{nz + 1} {ny + 1} {nx + 1}"/>\n',
           '      <Geometry GeometryType="VXVYVZ">\n']
    for fname, n in (("grid1D.bin", nx + 1), ("grid2D.bin", ny + 1), ("grid3D.bin", nz + 1)):
        out.append(f'        <DataItem Dimensions="{n}" NumberType="Float" Precision="8" Format="Binary" '
                   f'Endian="Little" Seek="{n * 8}">{fname}</DataItem>\n')
    out.append("      </Geometry>\n")
    for v, name in enumerate(NAMES):
        out.append(f'      <Attribute Name="{name}" AttributeType="Scalar" Center="Cell">\n')
        out.append(f'        <DataItem Dimensions="{nz} {ny} {nx}" NumberType="Float" Precision="8" '
                   f'Format="Binary" Endian="Little" Seek="{v * nx * ny * nz * 8}">{fdata}</DataItem>\n')
        out.append("      </Attribute>\n")
    out += ["    </Grid>\n", "  </Domain>\n", "</Xdmf>\n"]
    return "".join(out)


def ascii_snapshot(P: np.ndarray, x1a, x2a, x3a, nx: int, ny: int, time: float, dt: float) -> str:
    k = NGH
    x1b, x2b, x3b = centres(x1a), centres(x2a), centres(x3a)
    out = [f"# {time:.6e} {dt:.6e}\n", f"# {nx}\n", f"# {ny}\n", f"# {k} {x3b[k]:.6e}\n", "# x y d vx vy p X1\n"]
    for j in range(NGH, NGH + ny):
        for i in range(NGH, NGH + nx):
            vals = (x1b[i], x2b[j], P[k, j, 0, i], P[k, j, 1, i], P[k, j, 2, i], P[k, j, 5, i], P[k, j, 11, i])
            out.append(" ".join(f"{v:.6e}" for v in vals) + "\n")
        out.append("\n")
    return "".join(out)


def write_output(root: str, index: int, P: np.ndarray, axes, time: float, dt: float, ascii: bool = True) -> None:
    """Output(true) of the reference for one rank: every file, under root."""
    x1a, x2a, x3a = (np.asarray(a, dtype=np.float64) for a in axes)
    kt, jt, _, it = P.shape
    nx, ny, nz = it - 2 * NGH - 1, jt - 2 * NGH - 1, kt - 2 * NGH - 1
    b = os.path.join(root, "bindata")
    os.makedirs(b, exist_ok=True)
    with open(os.path.join(b, f"unf{index:05d}.dat"), "w") as f:
        f.write(f"# {time:.17g} {dt:.17g}\n# {nx} \n# {ny} \n# {nz} \n")
    for name, xa, n in (("grid1D.bin", x1a, nx), ("grid2D.bin", x2a, ny), ("grid3D.bin", x3a, nz)):
        grid_block(xa, n).astype("<f8").tofile(os.path.join(b, name))
    pack(P, nx, ny, nz).astype("<f8").tofile(os.path.join(b, f"field{index:05d}.bin"))
    with open(os.path.join(b, f"field{index:05d}.xmf"), "w") as f:
        f.write(xdmf(nx, ny, nz, time, index))
    if ascii:
        a = os.path.join(root, "ascdata")
        os.makedirs(a, exist_ok=True)
        with open(os.path.join(a, f"snap000-{index:05d}.csv"), "w") as f:
            f.write(ascii_snapshot(P, x1a, x2a, x3a, nx, ny, time, dt))
