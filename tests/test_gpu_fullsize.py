"""The benchmark workloads at their own sizes, checked through properties that
do not depend on the size: FP32-Kahan runs track FP64 twins, the bubble pair
stays mirror-symmetric, and every size class of the 96-run ensemble matches a
single lattice started from the same draw."""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import rel_err
from helpers import L

pytestmark = pytest.mark.gpu


def test_preheating_256_fp32_tracks_fp64(engine):
    """Two fields, 256^3, L = 10 pi, conformal, Yoshida-4, dt = dx/20, vacuum
    fluctuations: after 30 steps the FP32-Kahan run's P(k) (bins up to half
    the Nyquist wavenumber), a and energy follow the FP64 run."""
    n, length = 256, 10 * math.pi
    dt = length / n / 20
    out = {}
    for prec in (L.FP64, L.FP32_KAHAN):
        c = L.make_config(n, nfld=2, length=length, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                          precision=prec, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
        g = engine.Lattice(c)
        g.init_vacuum(1000, [1.0, 0.0], [0.0, 0.0], [3.0, 2.0], amp=1e-8)
        g.set_scale_factor(1.0, 0.0)
        g.calc_metric()
        g.symp(4, dt, 30)
        S = [g.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, 128)[0] for f in range(2)]
        out[prec] = (S, g.scale_factor(), g.energies())
        g.close()
    (S64, s64, e64), (S32, s32, e32) = out[L.FP64], out[L.FP32_KAHAN]
    for f in range(2):
        rel = np.abs(S32[f][1:64] - S64[f][1:64]) / np.abs(S64[f][1:64])
        assert rel.max() <= 1e-4, (f, rel.max())
    assert abs(s32[0] - s64[0]) <= 1e-8 * s64[0]
    assert abs(e32[L.E_RHO] - e64[L.E_RHO]) <= 1e-6 * abs(e64[L.E_RHO])


def test_bubbles_512_fp32_tracks_fp64_and_stays_symmetric(engine):
    """Two thin-wall bubbles 512^3, 27-point FD with GW sourcing, leapfrog:
    the FP32-Kahan fields follow the FP64 run, and the pair (mirror images
    about x = L/2) stays mirror-symmetric."""
    n = 512
    ln = n / 4.0
    res = {}
    for prec in (L.FP64, L.FP32_KAHAN):
        c = L.make_config(n, nfld=1, length=ln, laplacian=L.LAP_FD27, precision=prec, split_order=L.SPLIT_DEFROST,
                          model=L.MODEL_DOUBLE_WELL, model_params=(0.01,), gw=True, gw_coupling=2.0)
        g = engine.Lattice(c)
        g.init_bubbles([[0.34375 * ln, 0.5 * ln, 0.5 * ln], [0.65625 * ln, 0.5 * ln, 0.5 * ln]], 0.09375 * ln,
                       math.sqrt(2.0))
        g.symp(2, 0.025, 40)
        res[prec] = g.get_state()[0][0]
        g.close()
    f64, f32 = res[L.FP64], res[L.FP32_KAHAN]
    assert rel_err(f32, f64) <= 1e-5
    mirror = f32[:, :, (-np.arange(n)) % n]  # site i <-> n - i: x <-> L - x
    assert np.max(np.abs(mirror - f32)) <= 1e-5


def test_ensemble_96_runs_match_single_lattices(engine):
    """The 96-run FP32-Kahan ensemble (32 x 64^3, 32 x 96^3, 24 x 128^3,
    8 x 192^3) on the streamed passes: one run of every size class against an
    FP64 single lattice from the same draw.  The passes transform the field
    with its compensation, so the runs follow FP64 to the rounding of the
    Laplacian itself (a cuFFT FP32 lattice, which transforms the rounded
    field, differs from both by ~2e-5 of max |pi| after 10 steps)."""
    sizes = [64] * 32 + [96] * 32 + [128] * 24 + [192] * 8
    base = L.make_config(64, nfld=1, length=20.0, laplacian=L.LAP_SPECTRAL, precision=L.FP32_KAHAN,
                         model=L.MODEL_PHI4, model_params=(1.0,))
    ens = engine.Ensemble(base, sizes)
    seeds = list(range(5000, 5000 + len(sizes)))
    ens.init_vacuum(seeds, 1.0, 0.0, 3.0, amp=1e-8, kcut_frac=0.5)
    assert ens.sep_streamed()
    ens.symp(4, 1.0 / 20, 10)
    ens.sync()
    for r in (0, 33, 70, 95):
        n = sizes[r]
        c = L.make_config(n, nfld=1, length=20.0, laplacian=L.LAP_SPECTRAL, precision=L.FP64,
                          model=L.MODEL_PHI4, model_params=(1.0,))
        g = engine.Lattice(c)
        g.init_vacuum(seeds[r], [1.0], [0.0], [3.0], amp=1e-8, kcut_frac=0.5)
        g.symp(4, (20.0 / n) / 20, 10)
        f, p = g.get_state()
        ef, ep = ens.state(r)
        assert rel_err(ef, f[0]) <= 1e-5, (r, n, rel_err(ef, f[0]))
        assert rel_err(ep, p[0]) <= 1e-5, (r, n, rel_err(ep, p[0]))
        g.close()
    ens.close()
