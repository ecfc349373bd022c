"""Error-status contract of the C ABI on the GPU: a NaN in the uploaded state
is reported as LAT_ERR_NAN by the calls that read the lattice reductions, and
the handle is usable again after a fresh upload (the reference stops the
program on errors, hamiltonian_conformal.f90:77-79; the engine returns codes)."""
from __future__ import annotations

import math

import numpy as np
import pytest

from helpers import L, phi4_fd7, random_state, two_field_spectral

pytestmark = pytest.mark.gpu


def _nan_code(fn):
    with pytest.raises(L.LatticeError) as ei:
        fn()
    return ei.value.code


@pytest.mark.parametrize("case", ["spectral_fp64", "streamed_fp32", "fd7_fp64"])
def test_nan_upload_reports_and_handle_recovers(engine, case):
    if case == "fd7_fp64":
        c = phi4_fd7(16)
    else:
        prec = L.FP64 if case == "spectral_fp64" else L.FP32_KAHAN
        c = two_field_spectral(128 if case == "streamed_fp32" else 32, prec)
        if case == "streamed_fp32":
            c.spectral_impl = L.SPEC_IMPL_SEPARABLE
    g = engine.Lattice(c)
    if case == "streamed_fp32":
        assert g.sep_streamed()
    conf = c.background == L.BG_CONFORMAL
    f, p = random_state((g.nfld, g.nz, g.ny, g.nx), seed=5, mean=1.0, amp=0.02)
    dt = c.len / c.nx / 20

    def start(field):
        g.set_state(field, p)
        if conf:
            g.set_scale_factor(1.0, -0.1)

    start(f)
    e_ok = g.energies()
    bad = f.copy()
    bad[0, 3, 2, 1] = np.nan
    start(bad)
    assert _nan_code(g.energies) == 4  # LAT_ERR_NAN
    if conf:  # every conformal kick reduces the lattice sums of the Friedmann update
        g.symp(4, dt, 2)
        assert _nan_code(g.sync) == 4
        assert _nan_code(g.energies) == 4
    # a fresh upload clears the flag and the handle evolves as before
    start(f)
    e2 = g.energies()
    assert np.allclose(e2, e_ok, rtol=1e-12, atol=0)
    g.symp(4, dt, 2)
    g.sync()
    gf, _ = g.get_state()
    assert np.all(np.isfinite(gf))
    h = engine.Lattice(c)  # the same evolution on a handle that never saw the NaN
    h.set_state(f, p)
    if conf:
        h.set_scale_factor(1.0, -0.1)
    h.symp(4, dt, 2)
    hf, _ = h.get_state()
    assert np.max(np.abs(gf - hf)) <= (1e-13 if c.precision == L.FP64 else 1e-6) * np.max(np.abs(hf)), \
        np.max(np.abs(gf - hf))
    h.close()
    g.close()
