"""ctypes binding of the CPU oracle (oracle/liblatoracle.so).

TEST INFRASTRUCTURE ONLY: imported by the tests, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, to compare the engine against.  The engine never imports it.
Parity against the reference binary is unpinned (no Fortran compiler or FFTW
exists to build the reference); the oracle is pinned by analytic known-answer
tests and numpy.fft cross-checks instead.

State arrays are SoA float64 shaped (nfld, nz, ny, nx).
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "liblatoracle.so"
_lib = None


def _pkg():
    import importlib
    root = str(_HERE.parent)
    if root not in sys.path:
        sys.path.insert(0, root)
    return importlib.import_module("lattice-dev_gb300")


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        sys.path.insert(0, str(_HERE.parent / "lattice-dev_gb300"))
        from build import build_oracle  # noqa: E402
        build_oracle()
    lib = C.CDLL(str(LIB_PATH))
    P, D, I, U64 = C.c_void_p, C.c_double, C.c_int32, C.c_uint64
    dp = C.POINTER(C.c_double)
    cfgp = C.POINTER(_pkg().LatConfig)
    sig = {
        "orc_last_error": ([], C.c_char_p), "orc_create": ([C.POINTER(P), cfgp], I), "orc_destroy": ([P], I),
        "orc_set_state": ([P, dp, dp], I), "orc_get_state": ([P, dp, dp], I),
        "orc_gw_set": ([P, dp, dp], I), "orc_gw_get": ([P, dp, dp], I),
        "orc_set_scale_factor": ([P, D, D], I), "orc_get_scale_factor": ([P, dp, dp], I),
        "orc_get_time": ([P, dp], I), "orc_calc_metric": ([P], I), "orc_split": ([P, D, I], I),
        "orc_o2step": ([P, D, D, D], I), "orc_symp": ([P, I, D, I], I), "orc_laplacian": ([P, I, dp], I),
        "orc_energies": ([P, dp], I), "orc_spectrum_nbins": ([P, C.POINTER(I)], I),
        "orc_spectrum": ([P, I, I, I, I, dp, dp], I), "orc_crossspec": ([P, I, I, I, I, I, dp, dp], I),
        "orc_gw_spectrum": ([P, I, dp, dp], I), "orc_mode_gauss": ([U64, I, C.c_int64, dp], I),
        "orc_init_vacuum": ([P, U64, dp, dp, dp, D, D], I), "orc_init_bubbles": ([P, I, dp, D, D], I),
        "orc_init_sample": ([P, U64, dp, dp, D, D], I), "orc_rho_ball_sums": ([P, D, dp], I),
        "orc_fft_r2c_3d": ([I, I, I, dp, dp], I), "orc_fft_c2r_3d": ([I, I, I, dp, dp], I),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _check(code):
    if code != 0:
        raise RuntimeError(f"oracle status {code}: {_lib.orc_last_error().decode()}")


class Oracle:
    """CPU FP64 lattice with the same methods as the engine's Lattice."""

    def __init__(self, cfg):
        lib = load()
        self.cfg = cfg
        self._h = C.c_void_p()
        _check(lib.orc_create(C.byref(self._h), C.byref(cfg)))
        self.nx, self.ny, self.nz, self.nfld = cfg.nx, cfg.ny, cfg.nz, cfg.nfld

    def close(self):
        if self._h.value:
            _lib.orc_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self):
        return (self.nfld, self.nz, self.ny, self.nx)

    def set_state(self, fld, fldp=None):
        f = np.ascontiguousarray(np.asarray(fld, np.float64).reshape(self.shape()))
        p = None if fldp is None else np.ascontiguousarray(np.asarray(fldp, np.float64).reshape(self.shape()))
        _check(_lib.orc_set_state(self._h, _dp(f), _dp(p)))

    def get_state(self):
        f, p = np.empty(self.shape()), np.empty(self.shape())
        _check(_lib.orc_get_state(self._h, _dp(f), _dp(p)))
        return f, p

    def set_gw_state(self, u, pu):
        _check(_lib.orc_gw_set(self._h, _dp(np.ascontiguousarray(u, np.float64)), _dp(np.ascontiguousarray(pu, np.float64))))

    def gw_state(self):
        u = np.empty((6, self.nz, self.ny, self.nx))
        pu = np.empty_like(u)
        _check(_lib.orc_gw_get(self._h, _dp(u), _dp(pu)))
        return u, pu

    def set_scale_factor(self, a, ap):
        _check(_lib.orc_set_scale_factor(self._h, a, ap))

    def scale_factor(self):
        a, ap = C.c_double(), C.c_double()
        _check(_lib.orc_get_scale_factor(self._h, C.byref(a), C.byref(ap)))
        return a.value, ap.value

    def calc_metric(self):
        _check(_lib.orc_calc_metric(self._h))

    def symp(self, order, dt, nsteps):
        _check(_lib.orc_symp(self._h, order, dt, nsteps))

    def o2step(self, dt, w1, w2):
        _check(_lib.orc_o2step(self._h, dt, w1, w2))

    def hamiltonian_split(self, dt, hamind):
        _check(_lib.orc_split(self._h, dt, hamind))

    def time(self):
        t = np.zeros(3)
        _check(_lib.orc_get_time(self._h, _dp(t)))
        return t

    def laplacian(self, field=0):
        out = np.empty((self.nz, self.ny, self.nx))
        _check(_lib.orc_laplacian(self._h, field, _dp(out)))
        return out

    def energies(self):
        out = np.zeros(12)
        _check(_lib.orc_energies(self._h, _dp(out)))
        return out

    def nbins(self):
        ns = C.c_int32()
        _check(_lib.orc_spectrum_nbins(self._h, C.byref(ns)))
        return ns.value

    def spectrum(self, what=0, field=0, mode=0, nbins=None):
        nb = nbins or self.nbins()
        S, W = np.zeros(nb), np.zeros(nb)
        _check(_lib.orc_spectrum(self._h, what, field, mode, nb, _dp(S), _dp(W)))
        return S, W

    def crossspec_3d(self, what1, field1, what2, field2, nbins=None):
        nb = nbins or self.nbins()
        Sr, Si = np.zeros(nb), np.zeros(nb)
        _check(_lib.orc_crossspec(self._h, what1, field1, what2, field2, nb, _dp(Sr), _dp(Si)))
        return Sr, Si

    def gw_spectrum(self, nbins):
        S, W = np.zeros(nbins), np.zeros(nbins)
        _check(_lib.orc_gw_spectrum(self._h, nbins, _dp(S), _dp(W)))
        return S, W

    def init_vacuum(self, seed, fld0, dfld0, m2eff, amp=1e-8, kcut_frac=0.5):
        f0 = np.ascontiguousarray(np.broadcast_to(np.asarray(fld0, np.float64), (self.nfld,)))
        d0 = np.ascontiguousarray(np.broadcast_to(np.asarray(dfld0, np.float64), (self.nfld,)))
        m2 = np.ascontiguousarray(np.broadcast_to(np.asarray(m2eff, np.float64), (self.nfld,)))
        _check(_lib.orc_init_vacuum(self._h, C.c_uint64(seed), _dp(f0), _dp(d0), _dp(m2), amp, kcut_frac))

    def rho_ball_sums(self, r2=45.0):
        out = np.zeros(3)
        _check(_lib.orc_rho_ball_sums(self._h, float(r2), _dp(out)))
        return out

    def init_sample(self, seed, fld0, dfld0, m2eff, mpl=1e7 / 3):
        f0 = np.ascontiguousarray(np.broadcast_to(np.asarray(fld0, np.float64), (self.nfld,)))
        d0 = np.ascontiguousarray(np.broadcast_to(np.asarray(dfld0, np.float64), (self.nfld,)))
        _check(_lib.orc_init_sample(self._h, C.c_uint64(seed), _dp(f0), _dp(d0), float(m2eff), float(mpl)))

    def init_bubbles(self, centres, radius, width):
        c = np.ascontiguousarray(np.asarray(centres, np.float64).reshape(-1, 3))
        _check(_lib.orc_init_bubbles(self._h, c.shape[0], _dp(c), radius, width))


def fft_r2c_3d(f: np.ndarray) -> np.ndarray:
    load()
    f = np.ascontiguousarray(f, np.float64)
    nz, ny, nx = f.shape
    F = np.zeros((nz, ny, nx // 2 + 1), np.complex128)
    _check(_lib.orc_fft_r2c_3d(nx, ny, nz, _dp(f), F.ctypes.data_as(C.POINTER(C.c_double))))
    return F


def fft_c2r_3d(F: np.ndarray, nx: int) -> np.ndarray:
    load()
    F = np.ascontiguousarray(F, np.complex128).copy()
    nz, ny, _ = F.shape
    f = np.zeros((nz, ny, nx))
    _check(_lib.orc_fft_c2r_3d(nx, ny, nz, F.ctypes.data_as(C.POINTER(C.c_double)), _dp(f)))
    return f


def mode_gauss(seed: int, field: int, mode: int) -> tuple[float, float]:
    load()
    g = np.zeros(2)
    _check(_lib.orc_mode_gauss(C.c_uint64(seed), field, mode, _dp(g)))
    return float(g[0]), float(g[1])
