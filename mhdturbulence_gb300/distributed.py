"""The block-decomposed grid over processes: one block per rank, halos and reductions over
torch.distributed (NCCL between GPUs, gloo between hosts or for tests).

This is the multi-process form of the reference's MPI run: ranks in the row-major Cartesian order of
MPI_Cart_create (src_cpp_kokkos_host/mpi_config.cpp:61-69), the 2-deep primitive halos of the faces
shared with neighbours swapped after every step (SendRecvBoundary, boundary.cpp:222-318, 430-475,
627-672, MPI_Waitall at :715), and dt / c_h reduced over all ranks (MPIminfind / MPImaxfind,
mpi_config.cpp:83-99).  Blocks take their cell faces from the whole grid, so the decomposed run
equals the single-grid run bit for bit.

A rank's block is any object with the block interface (GpuBlock here: a Solver on this rank's GPU):
    coords, ntiles, bc, offset, extent, cfl, halo_dtype
    prepare()        recover P from U, fill the ghosts of non-exchanged faces, reduce dt / c_h locally
    step()           one step with the pending (global) dt / c_h, ending as prepare() does
    pack(face)       the 2 interior layers next to `face` (a tensor on the transport's device)
    recv_buffer(face)  (optional) an empty tensor that unpack(face, .) takes without a copy
    unpack(face, t)  into the 2 ghost layers beyond `face`
    get_reduction() / set_reduction(dtmin, chmax)   the pending reduction (dt = cfl * dtmin)
    sync()           a Report (step, time, dt, c_h, status)
"""
from __future__ import annotations

import numpy as np

from . import ic
from ._lib import BC_EXCHANGE
from .domain import block_bc, cart_coords, cart_rank, neighbour, split_axis


def block_geometry(nx, ny, nz, ntiles, coords):
    """(offset, extent) of the block at coords: first interior cell in the whole grid and cells per axis."""
    oe = [split_axis(n, t, c) for n, t, c in zip((nx, ny, nz), ntiles, coords)]
    return tuple(o for o, _ in oe), tuple(e for _, e in oe)


def sliced_axes(nx, ny, nz, domain, offset, extent):
    """The block's cell faces, taken from the whole grid's faces (length extent + 5 per axis)."""
    whole = ic.grid(nx, ny, nz, domain)
    return tuple(np.ascontiguousarray(a[o:o + e + 5]) for a, o, e in zip(whole, offset, extent))


class GpuBlock:
    """A block on this rank's GPU: a Solver with the block's extent, boundary kinds and faces.
    transport: "cuda" (halos as CUDA tensors, for NCCL) or "cpu" (page-locked host tensors that the
    halo kernels write and read over the host link, for gloo)."""

    def __init__(self, nx, ny, nz, ntiles, coords, domain=ic.KH_DOMAIN, bc=ic.KH_BC, gam=5.0 / 3.0, cfl=0.05,
                 precision="fp64", device=0, transport="cuda"):
        import torch

        from .solver import Solver
        self.coords, self.ntiles = tuple(coords), tuple(ntiles)
        self.offset, self.extent = block_geometry(nx, ny, nz, ntiles, coords)
        self.bc = block_bc(bc, ntiles, coords)
        self.cfl = cfl
        self.solver = Solver(*self.extent, domain=domain, bc=self.bc, gam=gam, cfl=cfl, precision=precision,
                             device=device)
        self.solver.set_grid(*sliced_axes(nx, ny, nz, domain, self.offset, self.extent))
        self.halo_dtype = torch.float32 if precision == "mixed" else torch.float64
        self.transport = transport
        self.device = device
        self.whole = (nx, ny, nz)

    def _buffer(self, face):
        import torch
        n = self.solver.halo_bytes(face) // (4 if self.halo_dtype == torch.float32 else 8)
        if self.transport == "cuda":
            return torch.empty(n, dtype=self.halo_dtype, device=f"cuda:{self.device}")
        return torch.empty(n, dtype=self.halo_dtype, pin_memory=True)

    def upload_cons(self, U):
        self.solver.upload_cons(U)

    def download_cons(self):
        return self.solver.download_cons()

    def init_kh_from_whole(self, U_whole):
        """Upload the block's part of a whole-grid conserved array."""
        o, e = self.offset, self.extent
        self.upload_cons(np.array(U_whole[o[2]:o[2] + e[2] + 5, o[1]:o[1] + e[1] + 5, :, o[0]:o[0] + e[0] + 5],
                                  copy=True))

    def init_kh(self, seed=1, **kw):
        """The block's part of the whole grid's KH state, made on the device (mhdgb_init_kh_block)."""
        self.solver.init_kh_block(self.whole, self.offset, seed=seed, **kw)

    def prepare(self):
        self.solver.prepare()

    def step(self):
        self.solver.step(1)

    def pack(self, face):
        import torch
        t = self._buffer(face)
        if self.transport == "cuda":
            torch.cuda.current_stream(self.device).synchronize()  # the buffer exists before the library writes it
        self.solver.halo_pack(face, t.data_ptr())
        return t

    def recv_buffer(self, face):
        return self._buffer(face)

    def unpack(self, face, t):
        import torch
        if self.transport == "cuda":
            torch.cuda.current_stream(self.device).synchronize()  # the received data has landed
        elif not t.is_pinned():
            t = t.pin_memory()
        self.solver.halo_unpack(face, t.data_ptr())

    def get_reduction(self):
        return self.solver.get_reduction()

    def set_reduction(self, dtmin, chmax):
        self.solver.set_reduction(dtmin, chmax)

    def sync(self):
        return self.solver.sync()


class DistributedGrid:
    """This rank's block of a decomposed grid, stepped in lockstep with the other ranks."""

    def __init__(self, block, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.block = block
        self.group = group
        self.rank = dist.get_rank(group)
        nt = block.ntiles
        if dist.get_world_size(group) != nt[0] * nt[1] * nt[2]:
            raise ValueError(f"{dist.get_world_size(group)} ranks for {nt[0]}x{nt[1]}x{nt[2]} blocks")
        if cart_coords(self.rank, nt) != tuple(block.coords):
            raise ValueError(f"rank {self.rank} holds block {block.coords}, expected {cart_coords(self.rank, nt)}")
        # (face, peer rank) of every exchanged face
        self.links = [(f, cart_rank(neighbour(block.coords, f, nt), nt)) for f in range(6)
                      if block.bc[f] == BC_EXCHANGE]

    def exchange(self):
        """Swap the halos of every exchanged face with the neighbours.  Sends go out in the order of
        this rank's faces and receives are posted in the order of the sending rank's faces (the face
        opposite the receiving one), so ranks that are neighbours across two faces (two blocks along
        a periodic axis) pair their messages correctly under ordered transports (NCCL) as well as
        tagged ones (gloo)."""
        import torch
        dist = self.dist
        sends = {f: self.block.pack(f) for f, _ in self.links}
        # page-locked for a host transport (empty_like of a page-locked tensor is pageable)
        alloc = getattr(self.block, "recv_buffer", None)
        recvs = {f: alloc(f) if alloc else torch.empty_like(sends[f]) for f, _ in self.links}
        ops = [dist.P2POp(dist.isend, sends[f], peer, self.group, tag=f) for f, peer in self.links]
        ops += [dist.P2POp(dist.irecv, recvs[f], peer, self.group, tag=f ^ 1)
                for f, peer in sorted(self.links, key=lambda fp: fp[0] ^ 1)]
        if ops:
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        for f, _ in self.links:
            self.block.unpack(f, recvs[f])

    def reduce(self):
        """dt and c_h over all ranks: min of the CFL time, max of the signal speed (both exact)."""
        import torch
        dist = self.dist
        dtmin, chmax = self.block.get_reduction()
        dev = "cpu" if getattr(self.block, "transport", "cpu") == "cpu" else f"cuda:{self.block.device}"
        t = torch.tensor([dtmin, -chmax], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MIN, group=self.group)
        self.block.set_reduction(float(t[0]), -float(t[1]))

    def prepare(self):
        self.block.prepare()
        self.exchange()
        self.reduce()

    def step(self, n=1):
        for _ in range(n):
            self.block.step()
            self.exchange()
            self.reduce()

    def sync(self):
        return self.block.sync()

    def gather_cons(self, nx, ny, nz):
        """The whole grid's conserved interior, assembled on rank 0 (None elsewhere)."""
        dist = self.dist
        U = self.block.download_cons()
        o, e = self.block.offset, self.block.extent
        part = (o, e, np.ascontiguousarray(U[2:2 + e[2], 2:2 + e[1], :, 2:2 + e[0]]))
        parts = [None] * dist.get_world_size(self.group) if self.rank == 0 else None
        dist.gather_object(part, parts, dst=0, group=self.group)
        if self.rank != 0:
            return None
        out = np.zeros((nz, ny, 10, nx))
        for (o, e, a) in parts:
            out[o[2]:o[2] + e[2], o[1]:o[1] + e[1], :, o[0]:o[0] + e[0]] = a
        return out


__all__ = ["DistributedGrid", "GpuBlock", "block_geometry", "sliced_axes"]
