"""CPU oracle pinned by golden vectors and analytic known-answer tests (no GPU).

The reference has no tests or fixtures and cannot be built here, so every pin
is either an exact enumeration of a quantity the reference defines, an
analytic solution of the discrete scheme, or an independent numerical
computation (numpy.fft, scipy's DOP853).
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_err
from helpers import L

GOLD = Path(__file__).resolve().parent / "golden"


def test_fft_matches_numpy(orc):
    rng = np.random.default_rng(0)
    for shape in [(4, 6, 8), (6, 10, 12), (5, 7, 9), (16, 16, 16), (30, 48, 96)]:
        f = rng.standard_normal(shape)
        F = orc.fft_r2c_3d(f)
        ref = np.fft.rfftn(f)
        assert rel_err(F, ref) < 1e-14
        g = orc.fft_c2r_3d(F, shape[2])
        assert rel_err(g / f.size, f) < 1e-14


def test_mode_counts_golden(orc):
    g = np.load(GOLD / "mode_counts.npz")
    for key in [k for k in g.files if k.startswith("W_")]:
        nx, ny, nz = map(int, key.split("_")[1:])
        if nx * ny * nz > 256 ** 3:
            continue  # 512^3: checked on the GPU machine (tests/test_gpu_benchsize.py), engine and oracle
        c = L.make_config((nx, ny, nz), nfld=1, length=1.0)
        o = orc.Oracle(c)
        assert o.nbins() == int(g[f"ns_{nx}_{ny}_{nz}"])
        o.set_state(np.random.default_rng(1).standard_normal((1, nz, ny, nx)))
        _, W = o.spectrum(0, 0, L.SPEC_COUNT)
        assert np.array_equal(W.astype(np.int64), g[key])


@pytest.mark.parametrize("lap,key", [(L.LAP_FD7, "fd7"), (L.LAP_FD27, "fd27"), (L.LAP_SPECTRAL, "spectral")])
def test_plane_wave_symbols(orc, lap, key):
    g = np.load(GOLD / "symbols.npz")
    n = int(g["n"])
    dx = 0.5
    c = L.make_config(n, nfld=1, length=n * dx, laplacian=lap)
    o = orc.Oracle(c)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    for m, sym in zip(g["m"], g[key]):
        f = np.cos(2 * np.pi * (m[0] * x + m[1] * y + m[2] * z) / n)
        o.set_state(f[None])
        lap_f = o.laplacian(0)
        assert np.max(np.abs(lap_f - sym / dx ** 2 * f)) <= 1e-11 * max(1.0, abs(sym) / dx ** 2)


def test_free_field_leapfrog_dispersion(orc):
    """A plane wave of V = m^2 phi^2/2 under symp2 follows phi_n = A cos(n theta),
    sin(theta/2) = (dt/2) sqrt(k_eff^2 + m^2), the exact solution of the discrete map."""
    n, dx, m2 = 16, 0.4, 3.0
    c = L.make_config(n, nfld=1, length=n * dx, laplacian=L.LAP_FD7, model=L.MODEL_FREE, model_params=(m2,))
    o = orc.Oracle(c)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    mvec = (2, 1, 3)
    f = 1e-3 * np.cos(2 * np.pi * (mvec[0] * x + mvec[1] * y + mvec[2] * z) / n)
    o.set_state(f[None], np.zeros_like(f)[None])
    keff2 = sum(4 / dx ** 2 * math.sin(math.pi * mi / n) ** 2 for mi in mvec)
    dt = dx / 10
    nsteps = 300
    o.symp(2, dt, nsteps)
    theta = 2 * math.asin(dt / 2 * math.sqrt(keff2 + m2))
    got = o.get_state()[0][0]
    assert np.max(np.abs(got - f * math.cos(nsteps * theta))) <= 1e-13


def _energy_drift(orc, order, dt, steps):
    n = 8
    c = L.make_config(n, nfld=1, length=8.0, laplacian=L.LAP_FD7, model=L.MODEL_PHI4)
    o = orc.Oracle(c)
    rng = np.random.default_rng(4)
    o.set_state(1.0 + 0.2 * rng.standard_normal((1, n, n, n)), 0.2 * rng.standard_normal((1, n, n, n)))
    e0 = o.energies()[L.E_RHO]
    worst = 0.0
    for _ in range(steps):
        o.symp(order, dt, 1)
        worst = max(worst, abs(o.energies()[L.E_RHO] - e0))
    return worst / abs(e0)


@pytest.mark.parametrize("order,expect", [(2, 4.0), (4, 16.0)])
def test_integrator_order(orc, order, expect):
    T = 2.0
    e1 = _energy_drift(orc, order, T / 20, 20)
    e2 = _energy_drift(orc, order, T / 40, 40)
    ratio = e1 / e2
    assert 0.7 * expect < ratio < 1.4 * expect, ratio


def test_homogeneous_phi4_vs_ode(orc):
    g = np.load(GOLD / "phi4_ode.npz")
    n = 4
    c = L.make_config(n, nfld=1, length=4.0, laplacian=L.LAP_SPECTRAL, model=L.MODEL_PHI4)
    o = orc.Oracle(c)
    o.set_state(np.ones((1, n, n, n)), np.zeros((1, n, n, n)))
    dt = 0.5 / 64
    t_prev = 0.0
    for t, phi in zip(g["t"][1:], g["phi"][1:]):
        o.symp(8, dt, int(round((t - t_prev) / dt)))
        t_prev = t
        assert abs(o.get_state()[0].mean() - phi) <= 1e-10


def test_energy_forms_agree(orc):
    for lap in (L.LAP_FD7, L.LAP_FD27):
        c = L.make_config(12, nfld=2, length=6.0, laplacian=lap, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
        o = orc.Oracle(c)
        rng = np.random.default_rng(2)
        o.set_state(rng.standard_normal((2, 12, 12, 12)), rng.standard_normal((2, 12, 12, 12)))
        e = o.energies()
        assert abs(e[L.E_GE_LAP] - e[L.E_GE_GRAD]) <= 1e-12 * abs(e[L.E_GE_LAP])


def test_friedmann_residual_bounded(orc):
    c = L.make_config(12, nfld=2, length=12.0, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                      model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    res = []
    for dt in (0.05, 0.025):
        o = orc.Oracle(c)
        o.init_vacuum(5, [1.0, 0.0], [0.0, 0.0], [3.0, 2.0], amp=1e-2, kcut_frac=0.5)
        o.calc_metric()
        assert abs(o.energies()[L.E_RESIDUAL]) < 1e-14
        o.symp(4, dt, int(round(2.0 / dt)))
        res.append(abs(o.energies()[L.E_RESIDUAL]))
    assert res[0] < 1e-5
    assert 8.0 < res[0] / res[1] < 32.0  # fourth order in dt


def test_rng_golden(orc):
    g = np.load(GOLD / "rng.npz")
    for key, gg in zip(g["keys"], g["gauss"]):
        got = orc.mode_gauss(int(key[0]), int(key[1]), int(key[2]))
        assert np.allclose(got, gg, rtol=1e-15, atol=1e-15)


def test_vacuum_statistics(orc):
    n = 32
    c = L.make_config(n, nfld=1, length=16.0, laplacian=L.LAP_SPECTRAL)
    o = orc.Oracle(c)
    amp, m2 = 1e-8, 3.0
    o.init_vacuum(11, [1.0], [0.0], [m2], amp=amp, kcut_frac=0.5)
    f, p = o.get_state()
    F = np.fft.rfftn(f[0] - 1.0)
    P = np.fft.rfftn(p[0])
    dk = 2 * np.pi / 16.0
    kx = np.arange(n // 2 + 1) * dk
    ky = np.fft.fftfreq(n, 1 / n) * dk
    K2 = kx[None, None, :] ** 2 + ky[None, :, None] ** 2 + ky[:, None, None] ** 2
    w = np.sqrt(K2 + m2)
    live = (K2 > 0) & (np.sqrt(K2) <= 0.5 * np.pi / 0.5)
    assert np.max(np.abs(F[~live])) <= 1e-12 * np.max(np.abs(F))
    # pi_k = -i w F_k for drawn modes, +i w F_k for their partners in the kx = 0 plane
    iz, iy, ix = np.meshgrid(np.arange(n), np.arange(n), np.arange(n // 2 + 1), indexing="ij")
    m = (iz * n + iy) * (n // 2 + 1) + ix
    mp = (((n - iz) % n) * n + (n - iy) % n) * (n // 2 + 1) + ix
    sign = np.where((ix == 0) & (mp < m), 1.0, -1.0)
    assert np.max(np.abs(P[live] - sign[live] * 1j * w[live] * F[live])) <= 1e-12 * np.max(np.abs(P))
    # <|F|^2> = amp N^2/(2 V w)
    V, N = 16.0 ** 3, n ** 3
    ratio = np.mean(np.abs(F[live]) ** 2 * 2 * V * w[live] / (amp * N ** 2))
    assert 0.9 < ratio < 1.1


def test_tt_projection(orc):
    n, dx = 12, 0.5
    c = L.make_config(n, nfld=1, length=n * dx, laplacian=L.LAP_FD7, gw=True, gw_coupling=1.0)
    o = orc.Oracle(c)
    rng = np.random.default_rng(8)
    f = rng.standard_normal((n, n, n))

    def D(g, ax):  # central difference: lattice momentum sin(k dx)/dx
        return (np.roll(g, -1, axis=ax) - np.roll(g, 1, axis=ax)) / (2 * dx)

    axes = {0: 2, 1: 1, 2: 0}  # component index -> array axis (x fastest)
    comps = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    # longitudinal (pure gauge) pi_ij = D_i D_j f and trace pi_ij = delta_ij f: no TT part
    long_ = np.stack([D(D(f, axes[i]), axes[j]) for i, j in comps])
    o.set_gw_state(np.zeros_like(long_), long_)
    S, W = o.gw_spectrum(12)
    ref = np.sum(long_ ** 2)
    assert np.max(np.abs(S * W)) <= 1e-20 * ref * n ** 6 + 1e-24
    trace = np.stack([f if i == j else 0 * f for i, j in comps])
    o.set_gw_state(np.zeros_like(trace), trace)
    S, W = o.gw_spectrum(12)
    assert np.max(np.abs(S)) <= 1e-20 * np.sum(f ** 2) * n ** 3
    # a transverse traceless wave along z: pi_12 = cos(k z) is its own TT part
    z = np.arange(n)[:, None, None] * np.ones((1, n, n))
    wave = np.zeros((6, n, n, n))
    wave[3] = np.cos(2 * np.pi * 2 * z / n)
    o.set_gw_state(np.zeros_like(wave), wave)
    S, W = o.gw_spectrum(12)
    total = np.sum(S * W)
    expect = 2 * np.sum(np.abs(np.fft.rfftn(wave[3])) ** 2 * np.where(np.arange(n // 2 + 1) == 0, 1, 2))
    assert abs(total - expect) <= 1e-12 * expect


def test_yoshida_weights_golden():
    g = np.load(GOLD / "yoshida.npz")
    w0, w1 = g["w4"]
    assert abs(w0 + 2 * w1 - 1) < 1e-15
    assert abs(2 * w1 ** 3 + w0 ** 3) < 1e-14  # third-order condition of the 4th-order composition


def _np_mode_gauss(seed, stream, modes):
    """The counter-based Box-Muller draw of orc_mode_gauss, in numpy uint64."""
    def mix(z):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))

    with np.errstate(over="ignore"):
        k0 = mix(mix(np.uint64(seed)) ^ np.uint64(stream))
        key = mix(k0 ^ modes.astype(np.uint64))
        u1 = ((mix(key ^ np.uint64(1)) >> np.uint64(11)).astype(np.float64) + 1.0) / 2.0 ** 53
        u2 = ((mix(key ^ np.uint64(2)) >> np.uint64(11)).astype(np.float64) + 1.0) / 2.0 ** 53
    r = np.sqrt(-2.0 * np.log(u1))
    return r * np.exp(2j * np.pi * u2)


def _np_sample(n, dx, seed, stream, gamma, m2eff, mpl):
    """sample(gamma, m2eff) of Pseudospec/openmp_dev/evolve_spectral.f90:421-506
    with scipy's DST-II (FFTW's RODFT10) and numpy FFTs; noise and the
    Hermitian projection of the kx = 0 and nx/2 planes as the oracle's."""
    from scipy import fft as sfft
    os_, nn = 16, n // 2 + 1
    nos = n * os_ * os_
    dk = 2 * np.pi / (n * dx)
    dxos, dkos, kcut = dx / os_, dk / (2 * os_), nn * dk / 2
    norm = 0.5 / (float(n) ** 3 * np.sqrt(2 * np.pi * dk ** 3) * mpl) * (dkos / dxos)
    kk = (np.arange(nos) + 0.5) * dkos
    ker = norm * sfft.dst(kk * (kk ** 2 + m2eff) ** gamma * np.exp(-(kk / kcut) ** 2), type=2) / np.arange(1, nos + 1)
    i = np.arange(n) + 1 - nn
    r = np.sqrt(i[None, None, :] ** 2 + i[None, :, None] ** 2 + i[:, None, None] ** 2) * os_
    l = np.floor(r).astype(np.int64)
    lo = ker[np.maximum(l, 1) - 1]
    f = np.where(l > 0, lo + (r - l) * (ker[np.minimum(l, nos - 1)] - lo), (4 * ker[0] - ker[1]) / 3)
    F = np.fft.rfftn(f)  # [z][y][x/2+1]
    F *= _np_mode_gauss(seed, stream, np.arange(F.size)).reshape(F.shape)
    for x in (0, n // 2):
        P = F[:, :, x]
        Q = np.conj(P[(-np.arange(n)) % n][:, (-np.arange(n)) % n])
        F[:, :, x] = 0.5 * (P + Q)
    return np.fft.irfftn(F, s=(n, n, n), axes=(0, 1, 2)) * n ** 3


@pytest.mark.parametrize("n", [8, 16])
def test_sample_ic_matches_numpy(orc, n):
    """The oracle's restatement of the reference's sample() IC (oversampled
    DST-II radial kernel, Box-Muller noise per mode) against scipy/numpy."""
    c = L.make_config(n, nfld=2, length=2.5 * n / 8, laplacian=L.LAP_SPECTRAL, model=L.MODEL_PHI4_G2,
                      model_params=(1.0, 2.0))
    o = orc.Oracle(c)
    fld0, dfld0, m2, mpl = [1.0, 0.2], [0.0, -0.1], 3.0, 0.5
    o.init_sample(1234, fld0, dfld0, m2, mpl)
    f, p = o.get_state()
    dx = c.len / n
    for l in range(2):
        wf = fld0[l] + _np_sample(n, dx, 1234, 0x5300 + 2 * l, -0.25, m2, mpl)
        wp = dfld0[l] + _np_sample(n, dx, 1234, 0x5300 + 2 * l + 1, 0.25, m2, mpl)
        assert np.max(np.abs(f[l] - wf)) <= 1e-9 * np.max(np.abs(wf - fld0[l]))
        assert np.max(np.abs(p[l] - wp)) <= 1e-9 * np.max(np.abs(wp - dfld0[l]))
        assert np.std(f[l]) > 0 and np.std(p[l]) > 0
