"""FP64 engine against the FP64 oracle at the benchmark lattices' own sizes.

* Two-field preheating, 256^3, L = 10 pi, pseudospectral Laplacian,
  self-consistent conformal expansion, Yoshida-4 with dt = dx/20, 100 steps
  from the seeded vacuum draw (Pseudospec/openmp_dev/evolve_spectral.f90:93-97,
  hamiltonian_conformal.f90:120-207): fields, momenta, a and ysclp of both
  FP64 spectral paths within 1e-10; the FP32-Kahan headline path within the
  stated FP32 tolerances of the same oracle run.
* Bubble collision with GW sourcing, 512^3, L = 128, 27-point stencil,
  leapfrog with dt = dx/10 (Discrete/Bubble-Collisions/evolve.f90:255-327):
  phi, pi, u_ij and pi_ij within 1e-10 after 10 steps, the TT spectrum of
  pi_ij within 1e-9 and its integer mode counts bit-exact.
* Integer shell mode counts (analysis_spec.f90:86-99,
  Discrete/Bubble-Collisions/analysis.f90:193-223) at 256^3 with 128 bins and
  512^3 with 256 bins, bit-exact against the brute-force enumeration in
  tests/golden/mode_counts.npz and against the oracle.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_err
from helpers import L

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
TOL64 = 1e-10


def preheating_cfg(prec, impl=0, n=256):
    return L.make_config(n, nfld=2, length=10 * math.pi, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                         precision=prec, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0), spectral_impl=impl)


def preheating_start(obj):
    obj.init_vacuum(1000, [1.0, 0.0], [0.0, 0.0], [3.0, 2.0], amp=1e-8, kcut_frac=0.5)
    obj.set_scale_factor(1.0, 0.0)
    obj.calc_metric()


def fluct_err(a, b):
    """Largest difference of the fluctuations (field minus its lattice mean)
    relative to the largest fluctuation of b, per field."""
    out = []
    for l in range(a.shape[0]):
        da = a[l] - b[l].mean()
        db = b[l] - b[l].mean()
        out.append(float(np.max(np.abs(da - db)) / np.max(np.abs(db))))
    return max(out)


def test_preheating_256_matches_oracle_100_steps(engine, orc):
    n = 256
    dt = 10 * math.pi / n / 20
    steps = 100
    o = orc.Oracle(preheating_cfg(L.FP64))
    preheating_start(o)
    of0, op0 = o.get_state()
    o.symp(4, dt, steps)
    of, op = o.get_state()
    oa, oap = o.scale_factor()
    oe = o.energies()
    nb = 128
    oS = [o.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, nb) for f in range(2)]
    oW = o.spectrum(L.SPEC_FLD, 0, L.SPEC_COUNT, nb)[1]
    o.close()
    counts = np.load(GOLD / "mode_counts.npz")["W_256_256_256"][:nb]
    assert np.array_equal(oW.astype(np.int64), counts)

    # both FP64 spectral paths: cuFFT and the separable passes
    for impl in (L.SPEC_IMPL_CUFFT, L.SPEC_IMPL_SEPARABLE):
        g = engine.Lattice(preheating_cfg(L.FP64, impl))
        preheating_start(g)
        gf0, gp0 = g.get_state()
        assert rel_err(gf0, of0) <= 1e-12 and rel_err(gp0, op0) <= 1e-12
        g.symp(4, dt, steps)
        gf, gp = g.get_state()
        ga, gap = g.scale_factor()
        ef, ep = rel_err(gf, of), rel_err(gp, op)
        print(f"impl {impl}: fields {ef:.2e} momenta {ep:.2e} fluct {fluct_err(gf, of):.2e} "
              f"a {abs(ga - oa) / oa:.2e} ap {abs(gap - oap) / abs(oap):.2e}")
        assert ef <= TOL64 and ep <= TOL64
        assert fluct_err(gf, of) <= 1e-9  # the fluctuations alone (~1e-5 of the mean field)
        assert abs(ga - oa) <= 1e-12 * oa and abs(gap - oap) <= TOL64 * abs(oap)
        for f in range(2):
            S, W = g.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, nb)
            assert rel_err(W, oS[f][1]) <= 1e-11  # smooth two-bin weights: FP64 sums of ~1e7 terms
            rel = np.abs(S[1:] - oS[f][0][1:]) / np.abs(oS[f][0][1:])
            assert rel.max() <= 1e-6, (f, rel.max())
        _, Wc = g.spectrum(L.SPEC_FLD, 0, L.SPEC_COUNT, nb)
        assert np.array_equal(Wc.astype(np.int64), counts)  # bit-exact integer mode counts
        ge = g.energies()
        assert abs(ge[L.E_RHO] - oe[L.E_RHO]) <= TOL64 * abs(oe[L.E_RHO])
        g.close()

    # the FP32-Kahan headline path (streamed separable passes) against the same FP64 oracle run
    g = engine.Lattice(preheating_cfg(L.FP32_KAHAN, L.SPEC_IMPL_SEPARABLE))
    preheating_start(g)
    assert g.sep_streamed()
    g.symp(4, dt, steps)
    ga, _ = g.scale_factor()
    ge = g.energies()
    for f in range(2):
        S, _ = g.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, nb)
        rel = np.abs(S[1:n // 4] - oS[f][0][1:n // 4]) / np.abs(oS[f][0][1:n // 4])
        print(f"fp32-kahan field {f}: P(k) max rel err up to k_Nyq/2 {rel.max():.2e}")
        assert rel.max() <= 1e-4, (f, rel.max())
    assert abs(ge[L.E_RHO] - oe[L.E_RHO]) <= 1e-6 * abs(oe[L.E_RHO])
    assert abs(ga - oa) <= 1e-8 * oa
    g.close()


def test_bubbles_512_fd27_gw_matches_oracle(engine, orc):
    n = 512
    ln = n / 4.0
    steps = 10
    c = L.make_config(n, nfld=1, length=ln, laplacian=L.LAP_FD27, precision=L.FP64, split_order=L.SPLIT_DEFROST,
                      model=L.MODEL_DOUBLE_WELL, model_params=(0.01,), gw=True, gw_coupling=2.0)
    centres = [[0.34375 * ln, 0.5 * ln, 0.5 * ln], [0.65625 * ln, 0.5 * ln, 0.5 * ln]]
    g = engine.Lattice(c)
    o = orc.Oracle(c)
    for obj in (g, o):
        obj.init_bubbles(centres, 0.09375 * ln, math.sqrt(2.0))
        obj.symp(2, 0.025, steps)
    gf, gp = g.get_state()
    of, op = o.get_state()
    assert rel_err(gf, of) <= TOL64 and rel_err(gp, op) <= TOL64
    del gf, gp, of, op
    gu, gpu_ = g.gw_state()
    ou, opu = o.gw_state()
    eu, epu = rel_err(gu, ou), rel_err(gpu_, opu)
    print(f"512^3 FD27+GW after {steps} steps: u {eu:.2e} pi_u {epu:.2e}")
    assert eu <= TOL64 and epu <= TOL64
    del gu, gpu_, ou, opu
    nb = 256
    Sg, Wg = g.gw_spectrum(nb)
    So, Wo = o.gw_spectrum(nb)
    counts = np.load(GOLD / "mode_counts.npz")["W_512_512_512"][:nb]
    assert np.array_equal(Wg.astype(np.int64), counts)
    assert np.array_equal(Wo.astype(np.int64), counts)
    assert rel_err(Sg, So) <= 1e-9, rel_err(Sg, So)
    g.close()
    o.close()


def test_mode_counts_512_exact(engine, orc):
    """Scalar-field spectra at 512^3 with 256 bins (SPEC_COUNT: the integer
    counts of spectrum_bin), the engine against the enumeration and the oracle."""
    n, nb = 512, 256
    c = L.make_config(n, nfld=1, length=128.0, laplacian=L.LAP_FD27, precision=L.FP32_KAHAN)
    g = engine.Lattice(c)
    o = orc.Oracle(L.make_config(n, nfld=1, length=128.0, laplacian=L.LAP_FD27))
    f = np.cos(2 * np.pi * 3 * np.arange(n) / n)[None, None, None, :] * np.ones((1, n, n, 1))
    g.set_state(f)
    o.set_state(f)
    del f
    counts = np.load(GOLD / "mode_counts.npz")["W_512_512_512"][:nb]
    Sg, Wg = g.spectrum(L.SPEC_FLD, 0, L.SPEC_COUNT, nb)
    So, Wo = o.spectrum(L.SPEC_FLD, 0, L.SPEC_COUNT, nb)
    assert np.array_equal(Wg.astype(np.int64), counts)
    assert np.array_equal(Wo.astype(np.int64), counts)
    assert rel_err(Sg, So) <= 1e-9
    g.close()
    o.close()
