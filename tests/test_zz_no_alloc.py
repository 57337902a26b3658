"""mhdgb_fill_ghosts_noalloc (the allocation-free ghost fill on a caller-owned device array) against
mhdgb_set_boundary, the handle-based SetBoundaryCondition, through the C ABI.

Tolerance: exact.  Both entry points only copy values or negate them, so the ghosts must agree bit
for bit, after one call and after a second call on the already-filled array (which then copies
the first call's edge ghosts).  The file is named to be collected last, so it also runs after every
other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

from mhdturbulence_gb300 import Solver, _lib

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

NPRIM = 12
CASES = [
    ((24, 16, 12), (1, 1, 2, 2, 1, 1), 0),   # the reference's KH boundaries, FieldArray layout
    ((9, 13, 7), (2, 3, 1, 1, 3, 2), 0),     # mixed types on every axis
    ((5, 4, 6), (3, 3, 3, 3, 2, 2), 3),      # padded rows (pitch = itot + 3)
    ((2, 2, 2), (2, 2, 2, 2, 2, 2), 8),      # the smallest grid, all reflecting
    ((40, 3, 2), (1, 1, 3, 3, 1, 1), 0),     # thin in y and z
]


def _fill(P, nx, ny, nz, pitch, bc, stream=None):
    bcs = (C.c_int * 6)(*bc)
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    return _lib.lib().mhdgb_fill_ghosts_noalloc(P.data_ptr(), nx, ny, nz, pitch, bcs, stream)


@pytest.mark.parametrize("shape,bc,pad", CASES)
def test_matches_set_boundary_on_two_calls_in_a_row(shape, bc, pad):
    nx, ny, nz = shape
    itot, jtot, ktot = nx + 5, ny + 5, nz + 5
    rng = np.random.default_rng(nx * 10007 + ny * 101 + nz)
    P0 = rng.standard_normal((ktot, jtot, NPRIM, itot)) + 2.0   # stale ghosts are random too

    with Solver(nx, ny, nz, bc=bc, precision="fp64_exact") as s:
        s.upload_prim(P0)
        s.SetBoundaryCondition()
        want1 = s.download_prim()
        s.SetBoundaryCondition()
        want2 = s.download_prim()
    assert not np.array_equal(want1, P0)

    pitch = itot + pad
    host = rng.standard_normal((ktot, jtot, NPRIM, pitch))
    host[..., :itot] = P0
    P = torch.from_numpy(host).to("cuda")
    rc = _fill(P, nx, ny, nz, pitch if pad else 0, bc)
    assert rc == 0, _lib.STATUS.get(rc, rc)
    torch.cuda.synchronize()
    got1 = P.cpu().numpy()
    rc = _fill(P, nx, ny, nz, pitch if pad else 0, bc)
    assert rc == 0, _lib.STATUS.get(rc, rc)
    torch.cuda.synchronize()
    got2 = P.cpu().numpy()

    assert np.array_equal(got1[..., :itot], want1)
    assert np.array_equal(got2[..., :itot], want2)
    assert np.array_equal(got2[..., itot:], host[..., itot:])   # row padding untouched


def test_on_a_caller_stream_without_allocating():
    """The use the entry point is for: a caller's own (non-default) stream, with the device's free
    memory the same before and after two calls.  Only that stream is synchronised before the
    result is read, so the two kernels of each call must run in order on it."""
    nx, ny, nz, bc = 20, 14, 10, (1, 1, 2, 2, 3, 1)
    itot, jtot, ktot = nx + 5, ny + 5, nz + 5
    rng = np.random.default_rng(7)
    P0 = rng.standard_normal((ktot, jtot, NPRIM, itot)) + 2.0
    with Solver(nx, ny, nz, bc=bc, precision="fp64_exact") as s:
        s.upload_prim(P0)
        s.SetBoundaryCondition()
        s.SetBoundaryCondition()
        want = s.download_prim()

    P = torch.from_numpy(P0).to("cuda")
    # the first call on a device loads the module, whose static scratch is then resident
    assert _fill(P, nx, ny, nz, 0, bc) == 0
    P.copy_(torch.from_numpy(P0))
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    assert _fill(P, nx, ny, nz, 0, bc, stream.cuda_stream) == 0
    assert _fill(P, nx, ny, nz, 0, bc, stream.cuda_stream) == 0
    stream.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    got = P.cpu().numpy()
    assert free_after == free_before
    assert np.array_equal(got, want)


def test_rejects_requests_it_cannot_serve():
    L = _lib.lib()
    P = torch.zeros((7, 7, NPRIM, 7), dtype=torch.float64, device="cuda")
    bc = (C.c_int * 6)(1, 1, 2, 2, 1, 1)
    # larger than the fixed scratch: rejected before the device is touched
    assert L.mhdgb_fill_ghosts_noalloc(P.data_ptr(), 2000, 500, 224, 0, bc, None) == -8
    assert L.mhdgb_status_string(-8).decode().startswith("grid too large")
    # invalid arguments
    assert L.mhdgb_fill_ghosts_noalloc(P.data_ptr(), 1, 2, 2, 0, bc, None) == -1
    assert L.mhdgb_fill_ghosts_noalloc(P.data_ptr(), 2, 2, 2, 6, bc, None) == -1   # pitch < itot
    assert L.mhdgb_fill_ghosts_noalloc(None, 2, 2, 2, 0, bc, None) == -1
    bad = (C.c_int * 6)(1, 1, 2, 2, 1, 4)
    assert L.mhdgb_fill_ghosts_noalloc(P.data_ptr(), 2, 2, 2, 0, bad, None) == -1
    host = np.zeros(7 * 7 * NPRIM * 7)
    assert L.mhdgb_fill_ghosts_noalloc(host.ctypes.data, 2, 2, 2, 0, bc, None) == -1   # not device memory
    # the array is untouched by every rejected call
    torch.cuda.synchronize()
    assert int(torch.count_nonzero(P)) == 0
