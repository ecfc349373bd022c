"""Energy conservation of the engine at the integrator's order.

The symplectic compositions of evolve_spectral.f90:129-227 conserve the
lattice energy up to an error of the integrator's order: halving dt over the
same time divides the energy drift by 2^order (4 for symp2, 16 for symp4).
The FP32-Kahan streamed passes must keep the energy (Minkowski) and the
Friedmann constraint (expanding background) within 1e-6 over the headline
model's first 100 steps.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from helpers import L, random_state

pytestmark = pytest.mark.gpu


def _drift(engine, order, dt, nsteps, prec=L.FP64, n=32):
    c = L.make_config(n, nfld=2, length=n * 0.5, laplacian=L.LAP_SPECTRAL, background=L.BG_MINKOWSKI,
                      precision=prec, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    g = engine.Lattice(c)
    f, p = random_state((2, n, n, n), seed=21, mean=1.0, amp=0.3)
    g.set_state(f, p)
    e0 = g.energies()[L.E_RHO]
    g.symp(order, dt, nsteps)
    e1 = g.energies()[L.E_RHO]
    g.close()
    return abs(e1 - e0) / abs(e0)


@pytest.mark.parametrize("order,expect", [(2, 4.0), (4, 16.0)])
def test_energy_error_scales_at_the_integrator_order(engine, order, expect):
    T = 2.0
    e1 = _drift(engine, order, T / 40, 40)
    e2 = _drift(engine, order, T / 80, 80)
    print(f"order {order}: drift {e1:.3e} -> {e2:.3e}, ratio {e1 / e2:.2f}")
    assert e1 > 1e-12  # the truncation error dominates FP64 rounding at these steps
    assert 0.7 * expect < e1 / e2 < 1.4 * expect, e1 / e2


def test_fp32_kahan_streamed_conserves_energy_and_friedmann(engine):
    n = 128
    length = 10 * math.pi * n / 256  # the headline model's spacing, dt = dx/20
    dt = length / n / 20
    # Minkowski: total energy
    c = L.make_config(n, nfld=2, length=length, laplacian=L.LAP_SPECTRAL, background=L.BG_MINKOWSKI,
                      precision=L.FP32_KAHAN, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0),
                      spectral_impl=L.SPEC_IMPL_SEPARABLE)
    g = engine.Lattice(c)
    assert g.sep_streamed()
    g.init_vacuum(1000, [1.0, 0.0], [0.0, 0.0], [3.0, 2.0], amp=1e-8, kcut_frac=0.5)
    e0 = g.energies()[L.E_RHO]
    g.symp(4, dt, 100)
    e1 = g.energies()[L.E_RHO]
    g.close()
    print(f"FP32-Kahan Minkowski energy change over 100 steps: {abs(e1 - e0) / e0:.2e}")
    assert abs(e1 - e0) <= 1e-6 * abs(e0)
    # expanding background: the Friedmann constraint residual (rho - 3H^2)/rho
    c = L.make_config(n, nfld=2, length=length, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                      precision=L.FP32_KAHAN, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0),
                      spectral_impl=L.SPEC_IMPL_SEPARABLE)
    g = engine.Lattice(c)
    g.init_vacuum(1000, [1.0, 0.0], [0.0, 0.0], [3.0, 2.0], amp=1e-8, kcut_frac=0.5)
    g.set_scale_factor(1.0, 0.0)
    g.calc_metric()
    g.symp(4, dt, 100)
    res = g.energies()[L.E_RESIDUAL]
    g.close()
    print(f"FP32-Kahan Friedmann residual after 100 steps: {res:.2e}")
    assert abs(res) <= 1e-6
