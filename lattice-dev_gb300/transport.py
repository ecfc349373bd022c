"""Multi-rank host logic for a decomposed lattice: transport, slabs, halos.

The reference distributes a lattice over MPI ranks: z-slabs with periodic
halo planes exchanged by MPI_Sendrecv before every FD kick
(Pseudospec/mpi_dev/hamiltonian_minkowski.f90:297-342,
Discrete/Bubble-Collisions/scafld.f90:120-192) and MPI_Allreduce of the
lattice sums that feed the Friedmann update (hamiltonian_conformal.f90:112-114,
198-201).  This module is that layer for GB300 machines: a ``Transport``
interface (implemented over torch.distributed: NCCL between GPUs, gloo between
CPU ranks for tests), a z-slab decomposition and the halo exchange.  On a
machine with one GPU the engine runs replicas; the exchange logic is
exercised by CPU ranks.
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
    """Transport over an initialised torch.distributed process group."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)

    def allreduce_sum(self, x: np.ndarray) -> np.ndarray:
        import torch
        t = torch.from_numpy(np.ascontiguousarray(x, np.float64).copy())
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
        return t.numpy()

    def sendrecv(self, send: np.ndarray, dest: int, recv: np.ndarray, src: int) -> None:
        import torch
        s = torch.from_numpy(np.ascontiguousarray(send, np.float64).copy())
        r = torch.empty(recv.shape, dtype=torch.float64)
        if self.size == 1:
            recv[...] = send
            return
        ops = [self.dist.P2POp(self.dist.isend, s, dest, self.group),
               self.dist.P2POp(self.dist.irecv, r, src, self.group)]
        for req in self.dist.batch_isend_irecv(ops):
            req.wait()
        recv[...] = r.numpy()

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
