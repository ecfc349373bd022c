"""Multi-rank halo exchange and reductions on CPU ranks (gloo, world size 2).

The distributed leapfrog on z-slabs must reproduce the single-domain oracle;
a lost peer must surface as an error on the surviving rank within the
process-group timeout instead of a hang.
"""
from __future__ import annotations

import datetime
import importlib
import os
import socket
import sys
import traceback
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _init(rank, size, port, timeout_s=60):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=size,
                            timeout=datetime.timedelta(seconds=timeout_s))
    return dist


def _leapfrog_worker(rank, size, port, fld, fldp, out_q):
    try:
        sys.path.insert(0, str(ROOT))
        T = importlib.import_module("lattice-dev_gb300.transport")
        dist = _init(rank, size, port)
        tr = T.TorchTransport()
        nz, ny, nx = fld.shape[1:]
        slab = T.decompose(nx, ny, nz, rank, size)
        f, p, tot = T.leapfrog_phi4(tr, slab, fld[:, slab.z0:slab.z1], fldp[:, slab.z0:slab.z1],
                                    dt=0.03, nsteps=6, dx=0.5)
        out_q.put((rank, slab.z0, slab.z1, f, p, tot))
        dist.barrier()
        dist.destroy_process_group()
    except Exception:  # noqa: BLE001
        out_q.put((rank, "error", traceback.format_exc()))


def test_slab_leapfrog_matches_oracle(orc):
    from helpers import L
    n = 8
    rng = np.random.default_rng(21)
    fld = 1.0 + 0.1 * rng.standard_normal((1, n, n, n))
    fldp = 0.1 * rng.standard_normal((1, n, n, n))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_leapfrog_worker, args=(r, 2, port, fld, fldp, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for pr in procs:
        pr.join(timeout=60)
    for r in res:
        assert r[1] != "error", r[2]
    f = np.zeros_like(fld)
    p = np.zeros_like(fldp)
    for rank, z0, z1, fs, ps, tot in res:
        f[:, z0:z1] = fs
        p[:, z0:z1] = ps
    o = orc.Oracle(L.make_config(n, nfld=1, length=n * 0.5, laplacian=L.LAP_FD7, model=L.MODEL_PHI4))
    o.set_state(fld, fldp)
    o.symp(2, 0.03, 6)
    of, op = o.get_state()
    assert np.max(np.abs(f - of)) <= 1e-13
    assert np.max(np.abs(p - op)) <= 1e-12
    ke, pe = res[0][5]
    assert abs(ke - np.sum(op * op)) <= 1e-12 * ke
    assert abs(pe - np.sum(0.25 * of ** 4)) <= 1e-12 * pe
    assert np.allclose(res[0][5], res[1][5], rtol=0, atol=0)  # every rank holds the same sums


def _lost_peer_worker(rank, size, port, out_q):
    try:
        dist = _init(rank, size, port, timeout_s=5)
        t = torch.ones(3, dtype=torch.float64)
        dist.all_reduce(t)  # both ranks join once
        if rank == 1:
            out_q.put((rank, "left"))
            out_q.close()
            out_q.join_thread()  # flush before leaving
            os._exit(0)  # leaves between steps, with nothing in flight
        try:
            dist.all_reduce(t)  # the Friedmann sums of the next substep
            out_q.put((rank, "no error"))
        except Exception as e:  # noqa: BLE001
            out_q.put((rank, "detected: " + type(e).__name__))
    except Exception:  # noqa: BLE001
        out_q.put((rank, "setup error " + traceback.format_exc()))


def test_lost_peer_is_detected():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_lost_peer_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = dict(q.get(timeout=120) for _ in range(2))
    for pr in procs:
        pr.join(timeout=60)
        if pr.is_alive():
            pr.kill()
    assert got[1] == "left"
    assert got[0].startswith("detected"), got[0]
