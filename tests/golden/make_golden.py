"""Generates the golden fixtures in tests/golden/ (run: python tests/golden/make_golden.py).

The reference lattice codes ship no tests, fixtures or golden vectors, and they
cannot be built here (Fortran + FFTW), so these vectors pin the oracle with
independent computations of quantities the reference defines exactly:

* ``mode_counts.npz`` -- integer shell mode counts of spectrum_bin
  (Discrete/Bubble-Collisions/analysis.f90:203-214) by brute-force enumeration
  of the reference loop (full x range, folded indices, l = floor(sqrt(m))+1),
  with math.isqrt (plane by plane in numpy for the 256^3 and 512^3 lattices
  of the benchmark workloads); also the bin count of init_spectrum_3d
  (Pseudospec/openmp_dev/analysis_spec.f90:55-56).
* ``symbols.npz`` -- the Fourier symbols of the 7- and 27-point stencils
  (Discrete/Bubble-Collisions/params.f90:116,119) and of the spectral
  Laplacian at a set of lattice momenta, evaluated in exact rational
  arithmetic for the cosines of multiples of 2 pi/n (via mpmath-free
  numpy float128 is not portable, so float64 is used and tolerances say so).
* ``phi4_ode.npz`` -- the homogeneous phi^4 oscillation phi'' = -phi^3,
  phi(0)=1, phi'(0)=0, from scipy's DOP853 at rtol 1e-13 (the oscillation the
  lattice's k = 0 mode must follow).
* ``rng.npz`` -- the first Gaussian pairs of the counter-based mode generator
  for fixed (seed, field, mode), computed here by an independent Python
  implementation of the published splitmix64 finaliser and Box-Muller.
* ``yoshida.npz`` -- the composition weights of symp4/6/8
  (Pseudospec/openmp_dev/evolve_spectral.f90:134-141,173-176,200-201).
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent
MASK = (1 << 64) - 1


def fold(i0, n):
    return i0 if i0 <= n // 2 else n - i0


def mode_counts(nx, ny, nz, nbins):
    W = np.zeros(nbins, np.int64)
    for k in range(nz):
        kk = fold(k, nz)
        for j in range(ny):
            jj = fold(j, ny)
            for i in range(nx):
                ii = fold(i, nx)
                l = math.isqrt(ii * ii + jj * jj + kk * kk)
                if l < nbins:
                    W[l] += 1
    return W


def mode_counts_planes(nx, ny, nz, nbins):
    """mode_counts enumerated one z-plane at a time with numpy integer
    arithmetic (the sizes of the benchmark lattices: 256^3 and 512^3)."""
    W = np.zeros(nbins, np.int64)
    ii = np.array([fold(i, nx) for i in range(nx)], np.int64)
    jj = np.array([fold(j, ny) for j in range(ny)], np.int64)
    r2 = ii[None, :] ** 2 + jj[:, None] ** 2
    for k in range(nz):
        kk = fold(k, nz)
        m = r2 + kk * kk
        l = np.floor(np.sqrt(m.astype(np.float64))).astype(np.int64)
        l -= (l * l > m)            # exact integer square root of m
        l += ((l + 1) * (l + 1) <= m)
        W += np.bincount(l[l < nbins].ravel(), minlength=nbins)[:nbins]
    return W


def ns_ref(nx, ny, nz):
    s = (nx // 2 + 1) ** 2 + (ny // 2 + 1) ** 2 + (nz // 2 + 1) ** 2
    return int(math.floor(math.sqrt(s + 1.0)))


def mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


def mode_gauss(seed, field, mode):
    key = mix64(mix64(mix64(seed) ^ field) ^ mode)
    u1 = ((mix64(key ^ 1) >> 11) + 1.0) * 2.0 ** -53
    u2 = ((mix64(key ^ 2) >> 11) + 1.0) * 2.0 ** -53
    r = math.sqrt(-2.0 * math.log(u1))
    th = 2 * math.pi * u2
    return r * math.cos(th), r * math.sin(th)


def main():
    shapes = [(8, 8, 8), (12, 10, 6), (16, 16, 16), (64, 64, 64), (24, 24, 24)]
    data = {}
    for s in shapes:
        nb = ns_ref(*s)
        data[f"W_{s[0]}_{s[1]}_{s[2]}"] = mode_counts(*s, nb)
        data[f"ns_{s[0]}_{s[1]}_{s[2]}"] = np.array(nb)
    for s in [(24, 24, 24), (64, 64, 64)]:  # the vectorised enumeration agrees with the loop
        assert np.array_equal(mode_counts_planes(*s, ns_ref(*s)), data[f"W_{s[0]}_{s[1]}_{s[2]}"])
    for s in [(256, 256, 256), (512, 512, 512)]:  # the two-field preheating and bubble lattices
        nb = ns_ref(*s)
        data[f"W_{s[0]}_{s[1]}_{s[2]}"] = mode_counts_planes(*s, nb)
        data[f"ns_{s[0]}_{s[1]}_{s[2]}"] = np.array(nb)
    np.savez_compressed(OUT / "mode_counts.npz", **data)

    n = 16
    ms = np.array([[1, 0, 0], [2, 3, 0], [4, 4, 4], [7, 1, 5], [8, 8, 8], [3, 5, 2]])
    th = 2 * np.pi * ms / n
    c = np.cos(th)
    s7 = -2 * np.sum(1 - c, axis=1)
    pairs = c[:, 0] * c[:, 1] + c[:, 0] * c[:, 2] + c[:, 1] * c[:, 2]
    s27 = (-128 + 28 * c.sum(1) + 12 * pairs + 8 * c.prod(1)) / 30
    spec = -np.sum((2 * np.pi * np.where(ms <= n // 2, ms, ms - n) / n) ** 2, axis=1)
    np.savez_compressed(OUT / "symbols.npz", n=n, m=ms, fd7=s7, fd27=s27, spectral=spec)

    from scipy.integrate import solve_ivp
    ts = np.linspace(0, 20, 41)
    sol = solve_ivp(lambda t, y: [y[1], -y[0] ** 3], (0, 20), [1.0, 0.0], method="DOP853", rtol=1e-13,
                    atol=1e-15, t_eval=ts)
    np.savez_compressed(OUT / "phi4_ode.npz", t=ts, phi=sol.y[0], pi=sol.y[1])

    keys = [(0, 0, 0), (1000, 0, 5), (1001, 1, 123456), (2 ** 40 + 3, 2, 99), (7, 0, 2 ** 31 - 1)]
    g = np.array([mode_gauss(*k) for k in keys])
    np.savez_compressed(OUT / "rng.npz", keys=np.array(keys, dtype=np.uint64), gauss=g)

    w1 = 1 / (2 - 2 ** (1 / 3))
    np.savez_compressed(OUT / "yoshida.npz", w4=np.array([1 - 2 * w1, w1]),
                        w6=np.array([0.784513610477560, 0.235573213359357, -1.177679984177887]),
                        w8=np.array([0.74167036435061295344822780, -0.40910082580003159399730010,
                                     0.19075471029623837995387626, -0.57386247111608226665638733,
                                     0.29906418130365592384446354, 0.33462491824529818378495798,
                                     0.31529309239676659663205666]))
    print("written to", OUT)


if __name__ == "__main__":
    main()
