"""Seeded initial conditions and the reference grid, as host arrays in the reference layout.

Arrays follow the reference FieldArray layout (src_cpp_kokkos_host/mhd.hpp:186-245,
``View(n1, nv, n2, n3)`` LayoutLeft): a C-ordered numpy array of shape ``(ktot, jtot, nv, itot)``
where ``itot = nx + 2*ngh + 1`` (src_cpp_kokkos_host/config.hpp:57-59) and ``ngh = 2``.

The grid follows GenerateGrid (src_cpp_kokkos_host/main.cpp:26-65): cell faces
``x1a(i) = dx*(i - (ngh+1)) + x1min`` and centres ``x1b(i) = (x1a(i+1)+x1a(i))/2``, i.e. the first
interior cell is centred at ``x1min - dx/2`` (the reference's ZEUS-style index offset is kept).

Random perturbations use a counter-based hash of (seed, global interior cell index), so a value
does not depend on how the domain is decomposed or on the platform.
"""
from __future__ import annotations

import numpy as np

NGH = 2
NPRIM = 12
NCONS = 10
# primitive indices (src_cpp_kokkos_host/mhd.hpp:250-253)
NDEN, NVE1, NVE2, NVE3, NENE, NPRE, NCSP, NBM1, NBM2, NBM3, NBPS, NST = range(12)
# conserved indices (src_cpp_kokkos_host/mhd.hpp:264-268)
MDEN, MRV1, MRV2, MRV3, METO, MBM1, MBM2, MBM3, MBPS, MST = range(10)

BC_PERIODIC, BC_REFLECTION, BC_OUTFLOW = 1, 2, 3
# The reference's default domain and boundaries (src_cpp_kokkos_host/config.hpp:21-38).
KH_DOMAIN = ((-0.5, 0.5), (-1.0, 1.0), (-0.5, 0.5))
KH_BC = (BC_PERIODIC, BC_PERIODIC, BC_REFLECTION, BC_REFLECTION, BC_PERIODIC, BC_PERIODIC)
CUBE_DOMAIN = ((-0.5, 0.5), (-0.5, 0.5), (-0.5, 0.5))
PERIODIC_BC = (BC_PERIODIC,) * 6


def extents(nx: int, ny: int, nz: int) -> tuple[int, int, int]:
    return nx + 2 * NGH + 1, ny + 2 * NGH + 1, nz + 2 * NGH + 1


def face_axis(n: int, lo: float, hi: float) -> np.ndarray:
    """Cell faces of one axis, GenerateGrid (main.cpp:35-44) for one rank."""
    xminloc = lo + (hi - lo) / 1 * 0
    xmaxloc = lo + (hi - lo) / 1 * (0 + 1)
    dx = (xmaxloc - xminloc) / float(n)
    i = np.arange(n + 2 * NGH + 1, dtype=np.float64)
    return dx * (i - (NGH + 1)) + xminloc


def grid(nx: int, ny: int, nz: int, domain=KH_DOMAIN):
    """Face coordinates (x1a, x2a, x3a) of the three axes."""
    return tuple(face_axis(n, lo, hi) for n, (lo, hi) in zip((nx, ny, nz), domain))


def centres(xa: np.ndarray) -> np.ndarray:
    xb = np.zeros_like(xa)
    xb[:-1] = 0.5 * (xa[1:] + xa[:-1])
    return xb


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def cell_uniform(seed: int, stream: int, shape_kji: tuple[int, int, int]) -> np.ndarray:
    """U[0,1) per interior cell from (seed, stream, global cell index); shape (nz, ny, nx)."""
    n = int(np.prod(shape_kji))
    idx = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + np.uint64(stream) * np.uint64(0x8CB92BA72F3D8DD7)
    h = _splitmix64(idx ^ _splitmix64(np.full(n, key, dtype=np.uint64)))
    return ((h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)).reshape(shape_kji)


def empty_field(nx: int, ny: int, nz: int, nv: int) -> np.ndarray:
    it, jt, kt = extents(nx, ny, nz)
    return np.zeros((kt, jt, nv, it), dtype=np.float64)


def interior(a: np.ndarray) -> np.ndarray:
    """View of the interior cells: shape (nz, ny, nv, nx)."""
    return a[NGH:-NGH - 1, NGH:-NGH - 1, :, NGH:-NGH - 1]


def prim_to_cons(prim: dict, gam: float) -> np.ndarray:
    """Conserved variables from a dict of interior primitive fields, each of shape (nz, ny, nx).

    Keys: rho, vx, vy, vz, p, bx, by, bz, psi, X.  The specific internal energy is
    p / (rho (gam-1)); the reference's conversion is src_cpp_kokkos_host/main.cpp:157-183."""
    rho = prim["rho"]
    nz, ny, nx = rho.shape
    U = empty_field(nx, ny, nz, NCONS)
    Ui = interior(U)
    e = prim["p"] / (rho * (gam - 1.0))
    ekin = 0.5 * rho * (prim["vx"] ** 2 + prim["vy"] ** 2 + prim["vz"] ** 2)
    emag = 0.5 * (prim["bx"] ** 2 + prim["by"] ** 2 + prim["bz"] ** 2)
    Ui[:, :, MDEN, :] = rho
    Ui[:, :, MRV1, :] = rho * prim["vx"]
    Ui[:, :, MRV2, :] = rho * prim["vy"]
    Ui[:, :, MRV3, :] = rho * prim["vz"]
    Ui[:, :, METO, :] = rho * e + ekin + emag
    Ui[:, :, MBM1, :] = prim["bx"]
    Ui[:, :, MBM2, :] = prim["by"]
    Ui[:, :, MBM3, :] = prim["bz"]
    Ui[:, :, MBPS, :] = prim["psi"]
    Ui[:, :, MST, :] = rho * prim["X"]
    return U


def _mesh(nx, ny, nz, domain):
    x1a, x2a, x3a = grid(nx, ny, nz, domain)
    xb, yb, zb = (centres(a)[NGH:NGH + n] for a, n in zip((x1a, x2a, x3a), (nx, ny, nz)))
    z, y, x = np.meshgrid(zb, yb, xb, indexing="ij")
    return x, y, z


def kh_prim(nx, ny, nz, seed=1, vshear=0.5, width=0.05, bx=0.1, amp=1.0e-2, sig=0.2,
            noise=1.0e-4, rho=1.0, p=1.0, domain=KH_DOMAIN):
    """Single shear layer Kelvin-Helmholtz set-up:
    v_x = vshear*tanh(y/width), rho, p uniform, B = (bx, 0, 0),
    v_y = amp*sin(2 pi x)*exp(-(y/sig)^2) + noise*(2u-1) with u seeded per cell,
    passive scalar X = (1 + tanh(y/width))/2, psi = 0."""
    x, y, z = _mesh(nx, ny, nz, domain)
    u = cell_uniform(seed, 0, x.shape)
    th = np.tanh(y / width)
    one = np.ones_like(x)
    return {
        "rho": rho * one, "p": p * one,
        "vx": vshear * th,
        "vy": amp * np.sin(2.0 * np.pi * x) * np.exp(-(y / sig) ** 2) + noise * (2.0 * u - 1.0),
        "vz": 0.0 * one,
        "bx": bx * one, "by": 0.0 * one, "bz": 0.0 * one, "psi": 0.0 * one,
        "X": 0.5 * (1.0 + th),
    }


def ref_kh_prim(nx, ny, nz, domain=KH_DOMAIN):
    """The reference's own double shear layer (src_cpp_kokkos_host/main.cpp:72-153), B = 0."""
    x, y, z = _mesh(nx, ny, nz, domain)
    wid, dv, sig, rrv = 0.05, 2.0, 0.2, 1.0e-2
    tp, tm = np.tanh((y + 0.5) / wid), np.tanh((y - 0.5) / wid)
    (x2min, x2max), (x3min, x3max) = domain[1], domain[2]
    harm = dv * rrv * np.cos(6 * 2 * np.pi * (y - x2min) / (x2max - x2min)) \
        * np.cos(6 * 2 * np.pi * (z - x3min) / (x3max - x3min))
    one = np.ones_like(x)
    return {
        "rho": one, "p": one,
        "vx": 0.5 * dv * (tp - tm - 1.0) + harm,
        "vy": 1.0e-3 * np.sin(2.0 * np.pi * x) * (np.exp(-(y + 0.5) ** 2 / sig ** 2) + np.exp(-(y - 0.5) ** 2 / sig ** 2)),
        "vz": 0.0 * one, "bx": 0.0 * one, "by": 0.0 * one, "bz": 0.0 * one, "psi": 0.0 * one,
        "X": 0.5 * (tp - tm),
    }


def random_smooth_prim(nx, ny, nz, seed=3, domain=CUBE_DOMAIN, bamp=0.3, vamp=0.4):
    """A smooth, fully three-dimensional state with every field non-trivial (all B components,
    psi and the scalar), for stage tests and mixed boundaries."""
    x, y, z = _mesh(nx, ny, nz, domain)
    r = np.random.default_rng(seed).uniform(0, 2 * np.pi, size=16)
    tp = 2 * np.pi
    rho = 1.0 + 0.3 * np.sin(tp * x + r[0]) * np.cos(tp * y + r[1]) + 0.1 * np.sin(tp * z + r[2])
    return {
        "rho": rho,
        "p": 0.8 + 0.2 * np.cos(tp * (x + y) + r[3]) * np.sin(tp * z + r[4]),
        "vx": vamp * np.sin(tp * y + r[5]) + 0.1 * np.cos(tp * z + r[6]),
        "vy": vamp * np.sin(tp * z + r[7]) * np.cos(tp * x + r[8]),
        "vz": vamp * np.cos(tp * x + r[9]) - 0.05,
        "bx": 0.2 + bamp * np.sin(tp * z + r[10]),
        "by": bamp * np.cos(tp * x + r[11]),
        "bz": -0.1 + bamp * np.sin(tp * y + r[12]),
        "psi": 0.01 * np.sin(tp * (x + z) + r[13]),
        "X": 0.5 + 0.4 * np.sin(tp * y + r[14]) * np.cos(tp * z + r[15]),
    }


def _spectral_field(shape, seed, stream, kmin=1.0, kmax=8.0, slope=-2.0):
    """Real random-phase field with 3D power |f_k|^2 ~ k**slope on kmin<=|k|<=kmax, unit rms."""
    nz, ny, nx = shape
    kz = np.fft.fftfreq(nz) * nz
    ky = np.fft.fftfreq(ny) * ny
    kx = np.fft.rfftfreq(nx) * nx
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    k = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    rng = np.random.default_rng([seed, stream])
    phase = rng.uniform(0.0, 2.0 * np.pi, size=k.shape)
    amp = np.where((k >= kmin) & (k <= kmax), np.power(np.maximum(k, 1e-30), slope / 2.0), 0.0)
    f = np.fft.irfftn(amp * np.exp(1j * phase), s=shape, axes=(0, 1, 2))
    return f / np.sqrt(np.mean(f ** 2)), (KX, KY, KZ, amp, phase)


def turbulence_prim(n, seed=7, sigma_lnrho=0.3, vrms=0.5, b0=0.2, beta=10.0, p=1.0):
    """Decaying-turbulence set-up on an n^3 periodic cube: log-normal density (sigma of ln rho,
    mean 1), uniform p, random-phase velocity modes 1<=|k|<=8 with 3D power ~ k^-2 scaled to rms
    vrms, and B = (b0,0,0) + curl A with A from the same spectrum, scaled so 2p/<B^2> = beta."""
    shape = (n, n, n)
    g, _ = _spectral_field(shape, seed, 0)
    lnr = sigma_lnrho * g
    rho = np.exp(lnr)
    rho /= rho.mean()
    v = [_spectral_field(shape, seed, 1 + c)[0] for c in range(3)]
    vn = np.sqrt(np.mean(v[0] ** 2 + v[1] ** 2 + v[2] ** 2))
    v = [vrms * c / vn for c in v]
    # B fluctuation: curl of a random vector potential, computed spectrally.
    A_hat = []
    for c in range(3):
        a, (KX, KY, KZ, amp, phase) = _spectral_field(shape, seed, 10 + c)
        A_hat.append(np.fft.rfftn(a, axes=(0, 1, 2)))
    tp = 2.0 * np.pi  # unit box: k in cycles per box
    bxh = 1j * tp * (KY * A_hat[2] - KZ * A_hat[1])
    byh = 1j * tp * (KZ * A_hat[0] - KX * A_hat[2])
    bzh = 1j * tp * (KX * A_hat[1] - KY * A_hat[0])
    db = [np.fft.irfftn(h, s=shape, axes=(0, 1, 2)) for h in (bxh, byh, bzh)]
    b2_target = 2.0 * p / beta - b0 * b0
    dbn = np.sqrt(np.mean(db[0] ** 2 + db[1] ** 2 + db[2] ** 2))
    db = [c * np.sqrt(max(b2_target, 0.0)) / dbn for c in db]
    zero = np.zeros(shape)
    return {
        "rho": rho, "p": p + zero, "vx": v[0], "vy": v[1], "vz": v[2],
        "bx": b0 + db[0], "by": db[1], "bz": db[2], "psi": zero.copy(),
        "X": 0.5 + 0.5 * np.tanh(4.0 * g),
    }
