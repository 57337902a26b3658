"""mhdgb_step_host, the reference-facing call that takes the state from a host array and returns it
in one: with page-locked, mapped arrays the recovery pass reads U_in over the host link and the last
step writes U_out as it updates each cell; ordinary arrays go through a device staging copy.  Both
routes give the same state bit for bit, into a separate array or in place, and U_out's ghost cells
are U_in's."""
import numpy as np
import pytest

from mhdturbulence_gb300 import Solver

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

NX, NY, NZ = 37, 29, 33  # partial tiles in x and y


def _pinned(a):
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
    t.numpy()[...] = a
    return t


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_exact"])
@pytest.mark.parametrize("nsteps", [1, 3, 17])
def test_mapped_arrays_match_staged_copies(precision, nsteps):
    with Solver(NX, NY, NZ, precision=precision) as s:
        s.init_kh(seed=3)
        U0 = s.download_cons()
        staged = np.full_like(U0, np.nan)
        dt0, ch0 = s.step_host(U0.copy(), staged, nsteps)
        assert np.isfinite(staged).all()

        src, dst = _pinned(U0), _pinned(np.full_like(U0, np.nan))
        dt1, ch1 = s.step_host(src.numpy(), dst.numpy(), nsteps)
        assert np.array_equal(dst.numpy(), staged)
        assert np.array_equal(src.numpy(), U0)  # the input is only read
        assert (dt1, ch1) == (dt0, ch0)

        inplace = _pinned(U0)
        dt2, ch2 = s.step_host(inplace.numpy(), inplace.numpy(), nsteps)
        assert np.array_equal(inplace.numpy(), staged)
        assert (dt2, ch2) == (dt0, ch0)

        # the device state is the returned one: stepping on from it equals stepping on from the array
        s.step(2)
        after_device = s.download_cons()
        s.upload_cons(staged)
        s.step(2)
        assert np.array_equal(s.download_cons(), after_device)


def test_ghost_cells_of_a_separate_output_are_the_inputs():
    with Solver(NX, NY, NZ) as s:
        s.init_kh(seed=4)
        U0 = s.download_cons()
        U0[..., 0] = 7.0  # mark the ghost and extra-index cells of the i axis
        src, dst = _pinned(U0), _pinned(np.zeros_like(U0))
        s.step_host(src.numpy(), dst.numpy(), 1)
        assert np.array_equal(dst.numpy()[..., 0], U0[..., 0])


def test_overlapping_arrays_give_the_same_state():
    with Solver(NX, NY, NZ) as s:
        s.init_kh(seed=5)
        U0 = s.download_cons()
        ref = np.empty_like(U0)
        s.step_host(U0.copy(), ref, 1)
        n, k = U0.size, 1000
        buf = torch.empty(n + k, dtype=torch.float64, pin_memory=True)
        b = buf.numpy()
        b[:n] = U0.ravel()
        s.step_host(b[:n].reshape(U0.shape), b[k:k + n].reshape(U0.shape), 1)
        assert np.array_equal(b[k:k + n].reshape(U0.shape), ref)
