"""Energy conservation of the engine at the integrator's order.

The symplectic compositions of evolve_spectral.f90:129-227 conserve the
lattice energy up to an error of the integrator's order: halving dt over the
same time divides the energy drift by 2^order (4 for symp2, 16 for symp4).
The FP32-Kahan streamed passes must keep the energy (Minkowski) and the
Friedmann constraint (expanding background) within 1e-6 over the headline
model's first 100 steps, and a run split into several calls must follow one
call of the same steps.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import rel_err
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


def test_streamed_calls_chunked_match_one_call(engine):
    """The first kick of every call takes its coefficients from the momentum
    sum that starts the call, the later kicks from the previous kick's
    finalize: four calls of 3 steps follow one call of 12 steps to FP32
    rounding (the two sums of pi^2 differ only in their summation order),
    and a(t) to 1e-12."""
    n = 128
    length = 10 * math.pi * n / 256
    dt = length / n / 20
    c = L.make_config(n, nfld=2, length=length, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                      precision=L.FP32_KAHAN, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0),
                      spectral_impl=L.SPEC_IMPL_SEPARABLE)
    out = []
    for calls, steps in ((1, 12), (4, 3)):
        g = engine.Lattice(c)
        assert g.sep_streamed()
        f, p = random_state((2, n, n, n), seed=23, mean=1.0, amp=0.05)
        g.set_state(f, p)
        g.set_scale_factor(1.0, 0.0)
        g.calc_metric()
        for _ in range(calls):
            g.symp(4, dt, steps)
        out.append((g.get_state(), g.scale_factor()))
        g.close()
    ((f1, p1), (a1, ap1)), ((f4, p4), (a4, ap4)) = out
    print(f"chunked vs one call: fields {rel_err(f4, f1):.2e} momenta {rel_err(p4, p1):.2e} a {abs(a4 - a1) / a1:.2e}")
    assert rel_err(f4, f1) <= 1e-6 and rel_err(p4, p1) <= 1e-5
    assert abs(a4 - a1) <= 1e-12 * a1 and abs(ap4 - ap1) <= 1e-8 * abs(ap1)
