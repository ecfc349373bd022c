"""The engine's z-slab handles (lat_slab_create) against the single-domain engine.

Two ranks (gloo over 127.0.0.1, spawned processes) each hold one engine
slab of the same lattice on the one GPU and exchange ghost planes through
torch.distributed before every kick, as the reference's MPI slabs do
(Pseudospec/mpi_dev/hamiltonian_minkowski.f90:297-342); the conformal case
all-reduces the Friedmann sums of every drift and kick
(hamiltonian_conformal.f90:112-114,198-201).  No kernel waits on another
rank: the exchange runs on the host between launches.  The slabs must
reproduce the single-domain run: FP64 to 1e-13, FP32-Kahan to FP32 rounding.
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

from conftest import rel_err
from helpers import L

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


CASES = {
    # the bubble workload's method: 27-point stencil, GW sourcing, DEFROST split, leapfrog
    "fd27_gw_fp64": dict(cfg=dict(n=(24, 20, 32), nfld=1, length=6.0, laplacian=L.LAP_FD27, precision=L.FP64,
                                  split_order=L.SPLIT_DEFROST, model=L.MODEL_DOUBLE_WELL, model_params=(0.01,),
                                  gw=True, gw_coupling=2.0),
                         order=2, dt=0.025, steps=10, conf=False, tol=1e-13),
    "fd27_gw_fp32": dict(cfg=dict(n=(32, 16, 32), nfld=1, length=8.0, laplacian=L.LAP_FD27, precision=L.FP32_KAHAN,
                                  split_order=L.SPLIT_DEFROST, model=L.MODEL_DOUBLE_WELL, model_params=(0.01,),
                                  gw=True, gw_coupling=2.0),
                         order=2, dt=0.025, steps=10, conf=False, tol=1e-6),
    # two fields, 7-point stencil, self-consistent expansion, Yoshida-4
    "fd7_conformal_fp64": dict(cfg=dict(n=(16, 12, 20), nfld=2, length=8.0, laplacian=L.LAP_FD7, precision=L.FP64,
                                        background=L.BG_CONFORMAL, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0)),
                               order=4, dt=0.05, steps=4, conf=True, tol=1e-13),
}


def _state(case):
    c = CASES[case]["cfg"]
    nx, ny, nz = c["n"]
    nf = c["nfld"]
    rng = np.random.default_rng(11)
    mean = 0.0 if c["model"] == L.MODEL_DOUBLE_WELL else 1.0
    f = mean + 0.2 * rng.standard_normal((nf, nz, ny, nx))
    p = 0.2 * rng.standard_normal((nf, nz, ny, nx))
    u = 0.05 * rng.standard_normal((6, nz, ny, nx)) if c.get("gw") else None
    pu = 0.05 * rng.standard_normal((6, nz, ny, nx)) if c.get("gw") else None
    return f, p, u, pu


def _run(lat, case, f, p, u, pu):
    spec = CASES[case]
    lat.set_state(f, p)
    if u is not None:
        lat.set_gw_state(u, pu)
    if spec["conf"]:
        lat.set_scale_factor(1.0, 0.0)
        lat.calc_metric()  # the Friedmann constraint from the (all-reduced) energies
    lat.symp(spec["order"], spec["dt"], spec["steps"])
    out = {"state": lat.get_state(), "energies": lat.energies(), "a": lat.scale_factor()}
    if u is not None:
        out["gw"] = lat.gw_state()
    return out


def _slab_worker(rank, size, port, case, q):
    try:
        for pth in (str(ROOT), str(ROOT / "tests")):
            if pth not in sys.path:
                sys.path.insert(0, pth)
        import torch.distributed as dist
        os.environ["MASTER_ADDR"] = "127.0.0.1"
        os.environ["MASTER_PORT"] = str(port)
        dist.init_process_group("gloo", rank=rank, world_size=size, timeout=datetime.timedelta(seconds=120))
        Lk = importlib.import_module("lattice-dev_gb300")
        T = importlib.import_module("lattice-dev_gb300.transport")
        spec = CASES[case]
        c = Lk.make_config(**spec["cfg"])
        m = c.nz // size
        z0, z1 = rank * m, (rank + 1) * m
        lat = Lk.SlabLattice(c, z0, z1)
        tr = T.TorchTransport()
        lat.set_hooks(*T.engine_slab_hooks(tr, lat))
        f, p, u, pu = _state(case)
        cut = (lambda a: None if a is None else np.ascontiguousarray(a[:, z0:z1]))
        out = _run(lat, case, cut(f), cut(p), cut(u), cut(pu))
        q.put((rank, z0, z1, out))
        lat.close()
        dist.barrier()
        dist.destroy_process_group()
    except Exception:  # noqa: BLE001
        q.put((rank, "error", traceback.format_exc(), None))


def _slabs(case, size=2):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_slab_worker, args=(r, size, port, case, q)) for r in range(size)]
    for pr in procs:
        pr.start()
    res = [q.get(timeout=600) for _ in range(size)]
    for pr in procs:
        pr.join(timeout=120)
    for r in res:
        assert r[1] != "error", r[2]
    return sorted(res, key=lambda r: r[1])


@pytest.mark.parametrize("case", list(CASES))
def test_two_slabs_match_single_domain(engine, case):
    spec = CASES[case]
    res = _slabs(case)
    f, p, u, pu = _state(case)
    g = engine.Lattice(L.make_config(**spec["cfg"]))
    ref = _run(g, case, f, p, u, pu)
    g.close()
    tol = spec["tol"]
    fs = np.concatenate([r[3]["state"][0] for r in res], axis=1)
    ps = np.concatenate([r[3]["state"][1] for r in res], axis=1)
    print(f"{case}: fields {rel_err(fs, ref['state'][0]):.2e} momenta {rel_err(ps, ref['state'][1]):.2e}")
    assert rel_err(fs, ref["state"][0]) <= tol
    assert rel_err(ps, ref["state"][1]) <= tol
    if u is not None:
        us = np.concatenate([r[3]["gw"][0] for r in res], axis=1)
        pus = np.concatenate([r[3]["gw"][1] for r in res], axis=1)
        assert rel_err(us, ref["gw"][0]) <= tol
        assert rel_err(pus, ref["gw"][1]) <= tol
    for r in res:  # every slab reports the energies and scale factor of the whole lattice
        e = r[3]["energies"]
        for i in (L.E_KE, L.E_GE_LAP, L.E_PE, L.E_RHO):
            assert abs(e[i] - ref["energies"][i]) <= max(tol, 1e-12) * abs(ref["energies"][i]), (i, e[i])
        if spec["conf"]:
            (a, ap), (ar, apr) = r[3]["a"], ref["a"]
            assert abs(a - ar) <= 1e-12 * ar and abs(ap - apr) <= 1e-11 * abs(apr), (a, ar, ap, apr)


def test_single_slab_wraps_onto_itself(engine):
    """One slab holding every plane: its halo exchange sends its boundary
    planes to its own ghosts, which is the periodic wrap."""
    case = "fd27_gw_fp64"
    spec = CASES[case]
    c = L.make_config(**spec["cfg"])
    lat = engine.SlabLattice(c, 0, c.nz)
    nb = lat.halo_bytes()
    lo, hi = (torch.empty(nb, dtype=torch.uint8, device="cuda") for _ in range(2))

    def halo(s):
        s.halo(0, lo.data_ptr())
        s.halo(1, hi.data_ptr())
        s.halo(2, hi.data_ptr())
        s.halo(3, lo.data_ptr())

    lat.set_hooks(halo, lambda v: v)
    f, p, u, pu = _state(case)
    out = _run(lat, case, f, p, u, pu)
    lat.close()
    g = engine.Lattice(c)
    ref = _run(g, case, f, p, u, pu)
    g.close()
    assert rel_err(out["state"][0], ref["state"][0]) <= 1e-13
    assert rel_err(out["gw"][1], ref["gw"][1]) <= 1e-13
    assert abs(out["energies"][L.E_RHO] - ref["energies"][L.E_RHO]) <= 1e-12 * abs(ref["energies"][L.E_RHO])


def test_slab_refusals(engine):
    c = L.make_config(16, nfld=1, length=4.0, laplacian=L.LAP_SPECTRAL)
    with pytest.raises(engine.LatticeError):
        engine.SlabLattice(c, 0, 8)  # the spectral Laplacian has no distributed transform here
    c = L.make_config(16, nfld=1, length=4.0, laplacian=L.LAP_FD7)
    lat = engine.SlabLattice(c, 4, 12)
    with pytest.raises(engine.LatticeError) as ei:
        lat.symp(2, 0.01, 1)  # no hooks set
    assert ei.value.code == 6  # LAT_ERR_STATE
    with pytest.raises(engine.LatticeError) as ei:
        lat.spectrum(L.SPEC_FLD, 0, L.SPEC_WEIGHTED, 8)
    assert ei.value.code == 8  # LAT_ERR_UNSUPPORTED
    lat.close()
