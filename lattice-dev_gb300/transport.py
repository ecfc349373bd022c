"""Multi-rank host logic for a decomposed lattice: transport, slabs, halos.

The reference distributes a lattice over MPI ranks: z-slabs with periodic
halo planes exchanged by MPI_Sendrecv before every FD kick
(Pseudospec/mpi_dev/hamiltonian_minkowski.f90:297-342,
Discrete/Bubble-Collisions/scafld.f90:120-192) and MPI_Allreduce of the
lattice sums that feed the Friedmann update (hamiltonian_conformal.f90:112-114,
198-201).  This module is that layer for GB300 machines: a ``Transport``
interface (implemented over torch.distributed: NCCL between GPUs, gloo between
CPU ranks), a z-slab decomposition, the halo exchange of numpy slabs, and
``engine_slab_hooks``, which drives the CUDA engine's own z-slab handles
(``SlabLattice``, lat_slab_create) through a Transport: the engine packs its
boundary planes into device buffers and calls back for the exchange before
every kick and for the all-reduce of every conformal lattice sum.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


class Transport:
    """Point-to-point and collective operations on float64 host arrays."""

    rank: int
    size: int

    def allreduce_sum(self, x: np.ndarray) -> np.ndarray:  # pragma: no cover - interface
        raise NotImplementedError

    def sendrecv(self, send: np.ndarray, dest: int, recv: np.ndarray, src: int) -> None:  # pragma: no cover
        raise NotImplementedError

    def barrier(self) -> None:  # pragma: no cover
        raise NotImplementedError


class TorchTransport(Transport):
    """Transport over an initialised torch.distributed process group.

    NCCL moves CUDA tensors only: with an NCCL group every message is staged
    through this rank's current CUDA device (and host arrays are copied back);
    with gloo the messages stay on the host."""

    def __init__(self, group=None):
        import torch
        import torch.distributed as dist
        self.torch = torch
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)
        self.backend = str(dist.get_backend(group)).lower()
        self.device = (torch.device("cuda", torch.cuda.current_device()) if self.backend == "nccl"
                       else torch.device("cpu"))

    def _wire(self, x: np.ndarray):
        return self.torch.from_numpy(np.ascontiguousarray(x, np.float64).copy()).to(self.device)

    def allreduce_sum(self, x: np.ndarray) -> np.ndarray:
        t = self._wire(x)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        return t.cpu().numpy()

    def sendrecv(self, send: np.ndarray, dest: int, recv: np.ndarray, src: int) -> None:
        if self.size == 1:
            recv[...] = send
            return
        s = self._wire(send)
        r = self.torch.empty(recv.shape, dtype=self.torch.float64, device=self.device)
        self._p2p(s, dest, r, src)
        recv[...] = r.cpu().numpy()

    def sendrecv_tensor(self, send, dest: int, recv, src: int) -> None:
        """send/recv: torch tensors on any device; the transfer runs on the
        group's device (CUDA for NCCL, the host for gloo)."""
        if self.size == 1:
            recv.copy_(send)
            return
        s = send if send.device == self.device else send.to(self.device)
        r = recv if recv.device == self.device else self.torch.empty_like(recv, device=self.device)
        self._p2p(s, dest, r, src)
        if r is not recv:
            recv.copy_(r)

    def _p2p(self, s, dest, r, src):
        ops = [self.dist.P2POp(self.dist.isend, s, dest, self.group),
               self.dist.P2POp(self.dist.irecv, r, src, self.group)]
        for req in self.dist.batch_isend_irecv(ops):
            req.wait()
        if self.device.type == "cuda":
            self.torch.cuda.synchronize(self.device)

    def barrier(self) -> None:
        self.dist.barrier(self.group)


@dataclass
class Slab:
    """The z-planes [z0, z1) of an (nz, ny, nx) lattice owned by one rank."""

    rank: int
    size: int
    nx: int
    ny: int
    nz: int
    z0: int
    z1: int

    @property
    def nzl(self) -> int:
        return self.z1 - self.z0

    @property
    def up(self) -> int:
        return (self.rank + 1) % self.size

    @property
    def down(self) -> int:
        return (self.rank - 1) % self.size


def decompose(nx: int, ny: int, nz: int, rank: int, size: int) -> Slab:
    """Even z-slabs (the FFTW-MPI slab split, Pseudospec/mpi_dev/initialize.f90:69-106)."""
    if nz % size:
        raise ValueError("nz must be a multiple of the number of ranks")
    m = nz // size
    return Slab(rank, size, nx, ny, nz, rank * m, (rank + 1) * m)


def exchange_halo(tr: Transport, slab: Slab, f: np.ndarray) -> np.ndarray:
    """f: (nfld, nzl, ny, nx) slab interior; returns (nfld, nzl+2, ny, nx) with one
    periodic ghost plane below and above, as wrap_field does for the z direction."""
    nf = f.shape[0]
    g = np.empty((nf, slab.nzl + 2, slab.ny, slab.nx))
    g[:, 1:-1] = f
    # send the top plane up, receive the lower ghost from below; then the reverse
    recv = np.empty((nf, slab.ny, slab.nx))
    tr.sendrecv(f[:, -1], slab.up, recv, slab.down)
    g[:, 0] = recv
    tr.sendrecv(f[:, 0], slab.down, recv, slab.up)
    g[:, -1] = recv
    return g


def stencil_lap(g: np.ndarray, c: tuple[float, float, float, float], cc: float, dx: float) -> np.ndarray:
    """STENCIL(c, LAPLACE)/(cc dx^2) of the interior planes of a halo-padded slab;
    x and y wrap locally (they are not distributed)."""
    c0, c1, c2, c3 = c
    out = []
    for k in range(1, g.shape[1] - 1):
        r1 = r2 = r3 = 0.0
        for dz in (-1, 0, 1):
            pl = g[:, k + dz]
            for dy in (-1, 0, 1):
                for dxx in (-1, 0, 1):
                    rank = (dxx != 0) + (dy != 0) + (dz != 0)
                    if rank == 0:
                        continue
                    v = np.roll(np.roll(pl, -dy, axis=1), -dxx, axis=2)
                    if rank == 1:
                        r1 = r1 + v
                    elif rank == 2:
                        r2 = r2 + v
                    else:
                        r3 = r3 + v
        out.append((c0 * g[:, k] + c1 * r1 + c2 * r2 + c3 * r3) / (cc * dx * dx))
    return np.stack(out, axis=1)


def leapfrog_phi4(tr: Transport, slab: Slab, fld: np.ndarray, fldp: np.ndarray, dt: float, nsteps: int,
                  dx: float, c=(-6.0, 1.0, 0.0, 0.0), cc=1.0, lam=1.0):
    """symp2 of V = lam phi^4/4 on a z-slab: D(dt/2) [K(dt) D(dt)]^(n-1) K(dt) D(dt/2),
    one halo exchange per kick; returns the slab state and the global energy sums."""
    f = fld.copy()
    p = fldp.copy()
    f += 0.5 * dt * p
    for j in range(nsteps):
        g = exchange_halo(tr, slab, f)
        lap = stencil_lap(g, c, cc, dx)
        p += dt * (lap - lam * f ** 3)
        f += (dt if j < nsteps - 1 else 0.5 * dt) * p
    ke = np.sum(p * p)
    pe = np.sum(0.25 * lam * f ** 4)
    tot = tr.allreduce_sum(np.array([ke, pe]))
    return f, p, tot


def engine_slab_hooks(tr: Transport, lat, device=None):
    """Hooks (halo, allreduce) for an engine z-slab handle ``lat``
    (``SlabLattice``) whose ranks form a periodic ring in z: before every kick
    the highest interior plane goes to the rank above, whose lower ghost it
    fills, and the lowest to the rank below; lattice sums are all-reduced.
    The halo messages live in device buffers of ``lat_slab_halo_bytes``."""
    import torch
    dev = device if device is not None else torch.device("cuda", lat.cfg.device)
    nb = lat.halo_bytes()
    lo, hi, glo, ghi = (torch.empty(nb, dtype=torch.uint8, device=dev) for _ in range(4))
    up, down = (tr.rank + 1) % tr.size, (tr.rank - 1) % tr.size

    def halo(s):
        s.halo(0, lo.data_ptr())   # the call returns once the copy has completed
        s.halo(1, hi.data_ptr())
        tr.sendrecv_tensor(hi, up, glo, down)
        tr.sendrecv_tensor(lo, down, ghi, up)
        torch.cuda.synchronize(dev)  # the received planes are in place before the engine reads them
        s.halo(2, glo.data_ptr())
        s.halo(3, ghi.data_ptr())

    def allreduce(v: np.ndarray) -> np.ndarray:
        return tr.allreduce_sum(v)

    return halo, allreduce
