"""Configuration builders shared by the tests (sizes small enough for the oracle)."""
from __future__ import annotations

import importlib
import math

import numpy as np

L = importlib.import_module("lattice-dev_gb300")


def cfg(n, **kw):
    return L.make_config(n, **kw)


def phi4_fd7(n=16, prec=L.FP64, length=None):
    # the 64^3 plain-method workload scaled down: phi^4, Minkowski, 7-point FD
    return cfg(n, nfld=1, length=length or 20.0 * n / 64, laplacian=L.LAP_FD7, background=L.BG_MINKOWSKI,
               precision=prec, model=L.MODEL_PHI4, model_params=(1.0,))


def two_field_spectral(n=32, prec=L.FP64, conformal=True):
    # two-field preheating V = phi^4/4 + g2 phi^2 chi^2/2, g2 = 2, L = 10 pi (scaled)
    return cfg(n, nfld=2, length=10 * math.pi * n / 256 * 4, laplacian=L.LAP_SPECTRAL,
               background=L.BG_CONFORMAL if conformal else L.BG_MINKOWSKI, precision=prec,
               model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))


def bubble_fd27(n=24, prec=L.FP64, gw=True, split=L.SPLIT_DEFROST):
    return cfg(n, nfld=1, length=0.25 * n, laplacian=L.LAP_FD27, background=L.BG_MINKOWSKI, precision=prec,
               split_order=split, model=L.MODEL_DOUBLE_WELL, model_params=(0.01,), gw=gw, gw_coupling=2.0)


def vacuum_ic(obj, seed=7, fld0=1.0, m2=3.0, amp=1e-4):
    nf = obj.nfld
    f0 = [fld0] + [0.0] * (nf - 1)
    m2e = [m2] + [2.0] * (nf - 1)
    obj.init_vacuum(seed, f0, [0.0] * nf, m2e, amp=amp, kcut_frac=0.5)


def random_state(shape, seed=0, mean=1.0, amp=0.1):
    rng = np.random.default_rng(seed)
    f = mean + amp * rng.standard_normal(shape)
    p = amp * rng.standard_normal(shape)
    return f, p
