"""GB300 lattice engine: Python binding of the C ABI in include/lattice.h.

The class :class:`Lattice` mirrors the Fortran module procedures of the
reference lattice codes one to one:

=========================  ====================================================
reference routine          here
=========================  ====================================================
symp2/4/6/8(dt, nsteps)    ``Lattice.symp2(dt, n)`` ... ``Lattice.symp(order, dt, n)``
symp_o2step(dt, w1, w2)    ``Lattice.o2step(dt, w1, w2)``
Hamiltonian_Split(dt, i)   ``Lattice.hamiltonian_split(dt, i)``
laplacian_3d(...)          ``Lattice.laplacian(field)`` / :func:`laplacian_3d`
spectrum_3d(S, f, ...)     ``Lattice.spectrum_3d(what, field)`` / :func:`spectrum_3d`
spectrum_bin(f, S)         ``Lattice.spectrum_bin(what, field)``
crossspec_3d(...)          ``Lattice.crossspec_3d(...)``
dump_rho / homlat          ``Lattice.energies()``
calc_metric                ``Lattice.calc_metric()``
get_scale_factor/hubble    ``Lattice.scale_factor()`` / ``Lattice.hubble()``
make/read_check_pt         ``Lattice.checkpoint_write/read``
=========================  ====================================================

Errors raise :class:`LatticeError` carrying the C status code.  There is no
CPU fallback: without the built CUDA library every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "liblattice.so"

# enums of include/lattice.h
LAP_SPECTRAL, LAP_FD7, LAP_FD27 = 1, 7, 27
BG_MINKOWSKI, BG_CONFORMAL = 0, 1
FP64, FP32_KAHAN = 0, 1
SPLIT_PSEUDOSPEC, SPLIT_DEFROST = 0, 1
MODEL_PHI4, MODEL_PHI4_G2, MODEL_DOUBLE_WELL, MODEL_FREE = 0, 1, 2, 3
SPEC_FLD, SPEC_FLDP = 0, 1
SPEC_WEIGHTED, SPEC_COUNT = 0, 1
SPEC_IMPL_AUTO, SPEC_IMPL_CUFFT, SPEC_IMPL_SEPARABLE = 0, 1, 2
UNITS_PROGRAM, UNITS_CONFORMAL = 0, 1  # closure variables (lat_closure_units)
E_KE, E_GE_LAP, E_GE_GRAD, E_PE, E_RHO, E_GRAV, E_RESIDUAL, E_A, E_AP, E_MEAN0, E_MEAN1, E_GW = range(12)
NENERGY = 12
K_KICKDRIFT, K_DRIFT, K_KICK, K_KMUL, K_FFT_R2C, K_FFT_C2R, K_GW, K_OTHER, K_SEP_X, K_SEP_Y, K_SEP_Z = range(11)
NKCLASS = 11
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_TIMEOUT", 4: "ERR_NAN", 5: "ERR_ALLOC",
          6: "ERR_STATE", 7: "ERR_IO", 8: "ERR_UNSUPPORTED"}


class LatticeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class LatConfig(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("nfld", C.c_int32),
                ("len", C.c_double), ("laplacian", C.c_int32), ("background", C.c_int32),
                ("precision", C.c_int32), ("split_order", C.c_int32), ("model", C.c_int32),
                ("gw", C.c_int32), ("model_params", C.c_double * 4), ("stencil", C.c_double * 5),
                ("gw_coupling", C.c_double), ("device", C.c_int32), ("spectral_impl", C.c_int32),
                ("reserved", C.c_int32 * 6)]


_lib = None

# hooks of a z-slab handle (lat_halo_fn, lat_sum_fn)
HALO_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.c_void_p)
SUM_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.POINTER(C.c_double), C.c_int32)


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads liblattice.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with __graft_entry__.build() "
                          "(the engine has no CPU fallback)")
    lib = C.CDLL(str(p))
    _declare(lib)
    if path is None:
        _lib = lib
    return lib


def _declare(lib: C.CDLL) -> None:
    P, D, I, I64, U64 = C.c_void_p, C.c_double, C.c_int32, C.c_int64, C.c_uint64
    dp = C.POINTER(C.c_double)
    sig = {
        "lat_last_error": ([], C.c_char_p), "lat_version": ([], C.c_char_p),
        "lat_create": ([C.POINTER(P), C.POINTER(LatConfig)], I), "lat_destroy": ([P], I),
        "lat_get_config": ([P, C.POINTER(LatConfig)], I),
        "lat_upload": ([P, dp, I, I, dp, I, I], I), "lat_download": ([P, dp, I, I, dp, I, I], I),
        "lat_set_scale_factor": ([P, D, D], I), "lat_get_scale_factor": ([P, dp, dp], I),
        "lat_calc_metric": ([P], I), "lat_symp": ([P, I, D, I], I), "lat_symp_prepare": ([P, I, D, I], I), "lat_o2step": ([P, D, D, D], I),
        "lat_split": ([P, D, I], I), "lat_get_time": ([P, dp], I), "lat_sync": ([P], I),
        "lat_laplacian": ([P, I, dp], I), "lat_laplacian_3d": ([I, I, I, dp, D], I),
        "lat_energies": ([P, dp], I), "lat_spectrum_nbins": ([P, C.POINTER(I)], I),
        "lat_spectrum": ([P, I, I, I, I, dp, dp], I), "lat_crossspec": ([P, I, I, I, I, I, dp, dp], I),
        "lat_spectrum_3d": ([I, I, I, dp, I, I, dp, dp], I),
        "lat_spectrum_noalloc": ([P, I, I, I, I, I, I, P, P], I),
        "lat_gw_spectrum": ([P, I, dp, dp], I), "lat_gw_download": ([P, dp, dp], I),
        "lat_gw_upload": ([P, dp, dp], I),
        "lat_init_vacuum": ([P, U64, dp, dp, dp, D, D], I), "lat_init_bubbles": ([P, I, dp, D, D], I),
        "lat_init_sample": ([P, U64, dp, dp, D, D], I),
        "lat_init_bubbles_boosted": ([P, I, C.POINTER(I), D, D, D, D], I),
        "lat_checkpoint_write": ([P, C.c_char_p, D, I], I),
        "lat_checkpoint_read": ([P, C.c_char_p, dp, C.POINTER(I)], I),
        "lat_ens_create": ([C.POINTER(P), C.POINTER(LatConfig), I, C.POINTER(I)], I),
        "lat_ens_destroy": ([P], I), "lat_ens_init_vacuum": ([P, C.POINTER(U64), D, D, D, D, D], I),
        "lat_ens_symp": ([P, I, D, I], I), "lat_ens_energies": ([P, dp], I),
        "lat_ens_spectrum": ([P, I, I, dp, dp], I), "lat_ens_download": ([P, I, dp, dp], I),
        "lat_ens_sync": ([P], I), "lat_ens_prepare": ([P, I, D, I], I), "lat_ens_mark": ([P, I], I),
        "lat_ens_mark_elapsed": ([P, I, I, dp], I), "lat_ens_launch_count": ([P, C.POINTER(I64)], I),
        "lat_ens_autotune": ([P, C.c_char_p], I), "lat_ens_tuning_get": ([P, C.POINTER(I)], I),
        "lat_ens_sep_streamed": ([P, C.POINTER(I)], I),
        "lat_timing_enable": ([P, I], I), "lat_timing_read": ([P, I, dp, C.POINTER(I64)], I),
        "lat_timing_reset": ([P], I), "lat_mark": ([P, I], I), "lat_mark_elapsed": ([P, I, I, dp], I), "lat_launch_count": ([P, C.POINTER(I64)], I),
        "lat_device_ptr": ([P, I, C.POINTER(P)], I), "lat_host_alloc": ([C.POINTER(P), C.c_size_t], I),
        "lat_host_free": ([P], I), "lat_autotune": ([P, C.c_char_p], I),
        "lat_tuning_get": ([P, C.POINTER(I)], I), "lat_sep_streamed": ([P, C.POINTER(I)], I),
        "lat_write_cube": ([P, I, I, I, C.c_char_p, C.c_char_p, I, C.c_double], I),
        "lat_dev_alloc": ([I, C.POINTER(P), C.c_size_t], I), "lat_dev_free": ([P], I),
        "lat_memcpy": ([P, P, C.c_size_t, I], I),
        "lat_net_nparams": ([], I64), "lat_net_create": ([C.POINTER(P), I, U64], I), "lat_net_destroy": ([P], I),
        "lat_net_get_params": ([P, C.POINTER(C.c_float), I64], I),
        "lat_net_set_params": ([P, C.POINTER(C.c_float), I64], I),
        "lat_net_set_norm": ([P, dp, dp, dp], I), "lat_net_get_norm": ([P, dp, dp, dp], I),
        "lat_net_forward": ([P, P, I64, C.POINTER(I), I, I, I, I, P], I),
        "lat_net_grad": ([P, P, I64, C.POINTER(I), I, I, I, I, dp, C.POINTER(C.c_float)], I),
        "lat_net_train_step": ([P, P, I64, C.POINTER(I), I, I, I, I, D, dp], I),
        "lat_net_launch_count": ([P], I64), "lat_net_time_forward": ([P, I, I, I, I, dp], I),
        "lat_write_energy_line": ([P, C.c_char_p, D], I), "lat_write_spectrum_block": ([P, C.c_char_p], I),
        "lat_write_log_line": ([P, C.c_char_p, D], I),
        "lat_closure_attach": ([P, P, I, I], I), "lat_coarsen": ([P, I, I, P], I),
        "lat_slab_create": ([C.POINTER(P), C.POINTER(LatConfig), I, I], I),
        "lat_slab_set_hooks": ([P, HALO_FN, SUM_FN, P], I),
        "lat_slab_halo_bytes": ([P, C.POINTER(C.c_size_t)], I), "lat_slab_halo": ([P, I, P], I),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = args
        fn.restype = res


def _check(code: int) -> None:
    if code != 0:
        msg = _lib.lat_last_error().decode() if _lib is not None else ""
        raise LatticeError(code, msg)


def _dp(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_config(n, nfld=1, length=1.0, laplacian=LAP_SPECTRAL, background=BG_MINKOWSKI, precision=FP64,
                split_order=SPLIT_PSEUDOSPEC, model=MODEL_PHI4, model_params=(1.0,), stencil=None,
                gw=False, gw_coupling=0.0, device=0, spectral_impl=SPEC_IMPL_AUTO) -> LatConfig:
    nx, ny, nz = (n, n, n) if np.isscalar(n) else tuple(n)
    c = LatConfig()
    c.nx, c.ny, c.nz, c.nfld, c.len = nx, ny, nz, nfld, float(length)
    c.laplacian, c.background, c.precision = laplacian, background, precision
    c.split_order, c.model, c.gw = split_order, model, int(bool(gw))
    for i, v in enumerate(model_params):
        c.model_params[i] = float(v)
    if stencil is not None:
        for i, v in enumerate(stencil):
            c.stencil[i] = float(v)
    c.gw_coupling = float(gw_coupling)
    c.device = device
    c.spectral_impl = spectral_impl
    return c


class Lattice:
    """One lattice resident on the GPU (a C-ABI handle)."""

    def __init__(self, cfg: LatConfig | None = None, **kw):
        lib = load_library()
        self.cfg = cfg if cfg is not None else make_config(**kw)
        self._h = C.c_void_p()
        _check(lib.lat_create(C.byref(self._h), C.byref(self.cfg)))
        self.nx, self.ny, self.nz, self.nfld = self.cfg.nx, self.cfg.ny, self.cfg.nz, self.cfg.nfld
        self.N = self.nx * self.ny * self.nz

    # lifecycle
    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib.lat_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # state (SoA numpy views [field][z][y][x]) ---------------------------------
    def set_state(self, fld: np.ndarray, fldp: np.ndarray | None = None) -> None:
        """fld/fldp as float64 arrays shaped (nfld, nz, ny, nx)."""
        f = np.ascontiguousarray(np.moveaxis(np.asarray(fld, np.float64).reshape(self.nfld, self.nz, self.ny, self.nx), 0, -1))
        p = None
        if fldp is not None:
            p = np.ascontiguousarray(np.moveaxis(np.asarray(fldp, np.float64).reshape(self.nfld, self.nz, self.ny, self.nx), 0, -1))
        _check(_lib.lat_upload(self._h, _dp(f), 0, 0, _dp(p), 0, 0))

    def get_state(self) -> tuple[np.ndarray, np.ndarray]:
        f = np.empty((self.nz, self.ny, self.nx, self.nfld))
        p = np.empty_like(f)
        _check(_lib.lat_download(self._h, _dp(f), 0, 0, _dp(p), 0, 0))
        return np.ascontiguousarray(np.moveaxis(f, -1, 0)), np.ascontiguousarray(np.moveaxis(p, -1, 0))

    def upload_fortran(self, fld, lo, hi, fldp, plo, phi) -> None:
        """Arrays in the Fortran layout fld(nfld, 1-lo:n+hi, ...) given as C-order (nz', ny', nx', nfld)."""
        _check(_lib.lat_upload(self._h, _dp(fld), lo, hi, _dp(fldp), plo, phi))

    def download_fortran(self, fld, lo, hi, fldp, plo, phi) -> None:
        _check(_lib.lat_download(self._h, _dp(fld), lo, hi, _dp(fldp), plo, phi))

    # scale factor -------------------------------------------------------------
    def set_scale_factor(self, a: float, ap: float) -> None:
        _check(_lib.lat_set_scale_factor(self._h, a, ap))

    def scale_factor(self) -> tuple[float, float]:
        a, ap = C.c_double(), C.c_double()
        _check(_lib.lat_get_scale_factor(self._h, C.byref(a), C.byref(ap)))
        return a.value, ap.value

    def hubble(self) -> float:
        a, ap = self.scale_factor()
        return -ap / 6.0 / a ** 2

    def calc_metric(self) -> None:
        _check(_lib.lat_calc_metric(self._h))

    # integrator ----------------------------------------------------------------
    def symp(self, order: int, dt: float, nsteps: int) -> None:
        _check(_lib.lat_symp(self._h, order, dt, nsteps))

    def prepare_symp(self, order: int, dt: float, nsteps: int) -> None:
        """Capture (not run) the CUDA graph of symp(order, dt, nsteps)."""
        _check(_lib.lat_symp_prepare(self._h, order, dt, nsteps))

    def symp2(self, dt, nsteps):
        self.symp(2, dt, nsteps)

    def symp4(self, dt, nsteps):
        self.symp(4, dt, nsteps)

    def symp6(self, dt, nsteps):
        self.symp(6, dt, nsteps)

    def symp8(self, dt, nsteps):
        self.symp(8, dt, nsteps)

    def o2step(self, dt, w1, w2) -> None:
        _check(_lib.lat_o2step(self._h, dt, w1, w2))

    def hamiltonian_split(self, dt, hamind) -> None:
        _check(_lib.lat_split(self._h, dt, hamind))

    def time(self) -> np.ndarray:
        t = np.zeros(3)
        _check(_lib.lat_get_time(self._h, _dp(t)))
        return t

    def sync(self) -> None:
        _check(_lib.lat_sync(self._h))

    # analysis ------------------------------------------------------------------
    def laplacian(self, field: int = 0) -> np.ndarray:
        out = np.empty((self.nz, self.ny, self.nx))
        _check(_lib.lat_laplacian(self._h, field, _dp(out)))
        return out

    def energies(self) -> np.ndarray:
        out = np.zeros(NENERGY)
        _check(_lib.lat_energies(self._h, _dp(out)))
        return out

    def nbins(self) -> int:
        ns = C.c_int32()
        _check(_lib.lat_spectrum_nbins(self._h, C.byref(ns)))
        return ns.value

    def spectrum(self, what=SPEC_FLD, field=0, mode=SPEC_WEIGHTED, nbins=None):
        nb = nbins or self.nbins()
        S, W = np.zeros(nb), np.zeros(nb)
        _check(_lib.lat_spectrum(self._h, what, field, mode, nb, _dp(S), _dp(W)))
        return S, W

    def spectrum_3d(self, what=SPEC_FLD, field=0, nbins=None):
        return self.spectrum(what, field, SPEC_WEIGHTED, nbins)[0]

    def spectrum_bin(self, what=SPEC_FLD, field=0, nbins=None):
        return self.spectrum(what, field, SPEC_COUNT, nbins)

    def crossspec_3d(self, what1, field1, what2, field2, nbins=None):
        nb = nbins or self.nbins()
        Sr, Si = np.zeros(nb), np.zeros(nb)
        _check(_lib.lat_crossspec(self._h, what1, field1, what2, field2, nb, _dp(Sr), _dp(Si)))
        return Sr, Si

    def gw_spectrum(self, nbins):
        S, W = np.zeros(nbins), np.zeros(nbins)
        _check(_lib.lat_gw_spectrum(self._h, nbins, _dp(S), _dp(W)))
        return S, W

    def gw_state(self):
        u = np.empty((6, self.nz, self.ny, self.nx))
        pu = np.empty_like(u)
        _check(_lib.lat_gw_download(self._h, _dp(u), _dp(pu)))
        return u, pu

    def set_gw_state(self, u, pu):
        u = np.ascontiguousarray(u, np.float64)
        pu = np.ascontiguousarray(pu, np.float64)
        _check(_lib.lat_gw_upload(self._h, _dp(u), _dp(pu)))

    # initial conditions --------------------------------------------------------
    def init_vacuum(self, seed, fld0, dfld0, m2eff, amp=1e-8, kcut_frac=0.5) -> None:
        f0 = np.ascontiguousarray(np.broadcast_to(np.asarray(fld0, np.float64), (self.nfld,)))
        d0 = np.ascontiguousarray(np.broadcast_to(np.asarray(dfld0, np.float64), (self.nfld,)))
        m2 = np.ascontiguousarray(np.broadcast_to(np.asarray(m2eff, np.float64), (self.nfld,)))
        _check(_lib.lat_init_vacuum(self._h, C.c_uint64(seed), _dp(f0), _dp(d0), _dp(m2), amp, kcut_frac))


    def init_sample(self, seed, fld0, dfld0, m2eff, mpl=1e7 / 3) -> None:
        """The reference's sample() initial fields (lat_init_sample)."""
        f0 = np.ascontiguousarray(np.broadcast_to(np.asarray(fld0, np.float64), (self.nfld,)))
        d0 = np.ascontiguousarray(np.broadcast_to(np.asarray(dfld0, np.float64), (self.nfld,)))
        _check(_lib.lat_init_sample(self._h, C.c_uint64(seed), _dp(f0), _dp(d0), float(m2eff), float(mpl)))
    def init_bubbles(self, centres, radius, width) -> None:
        c = np.ascontiguousarray(np.asarray(centres, np.float64).reshape(-1, 3))
        _check(_lib.lat_init_bubbles(self._h, c.shape[0], _dp(c), radius, width))

    # checkpoint ----------------------------------------------------------------
    def init_bubbles_boosted(self, centres, r0, t0, phi_false, phi_true) -> None:
        """Expanding-wall bubbles as the reference's initbubble builds them
        (centres: 1-based site indices (x, y, z) per bubble)."""
        c = np.ascontiguousarray(np.asarray(centres, dtype=np.int32).reshape(-1, 3))
        _check(_lib.lat_init_bubbles_boosted(self._h, len(c), c.ctypes.data_as(C.POINTER(C.c_int32)), r0, t0,
                                             phi_false, phi_true))

    def checkpoint_write(self, directory, time=0.0, frame=0) -> None:
        _check(_lib.lat_checkpoint_write(self._h, str(directory).encode(), time, frame))

    def checkpoint_read(self, directory) -> tuple[float, int]:
        t, fr = C.c_double(), C.c_int32()
        _check(_lib.lat_checkpoint_read(self._h, str(directory).encode(), C.byref(t), C.byref(fr)))
        return t.value, fr.value

    # measurement ---------------------------------------------------------------
    def timing(self, on: bool) -> None:
        _check(_lib.lat_timing_enable(self._h, int(on)))

    def timing_read(self, kclass: int) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_int64()
        _check(_lib.lat_timing_read(self._h, kclass, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def timing_reset(self) -> None:
        _check(_lib.lat_timing_reset(self._h))

    def mark(self, slot: int) -> None:
        _check(_lib.lat_mark(self._h, slot))

    def mark_elapsed(self, a: int, b: int) -> float:
        ms = C.c_double()
        _check(_lib.lat_mark_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        n = C.c_int64()
        _check(_lib.lat_launch_count(self._h, C.byref(n)))
        return n.value

    def device_ptr(self, what: int) -> int:
        p = C.c_void_p()
        _check(_lib.lat_device_ptr(self._h, what, C.byref(p)))
        return p.value or 0

    def autotune(self, cache_path=None) -> None:
        _check(_lib.lat_autotune(self._h, None if cache_path is None else str(cache_path).encode()))

    def tuning(self) -> list[int]:
        out = (C.c_int32 * 6)()
        _check(_lib.lat_tuning_get(self._h, out))
        return list(out)

    def sep_streamed(self) -> bool:
        on = C.c_int32()
        _check(_lib.lat_sep_streamed(self._h, C.byref(on)))
        return bool(on.value)

    # output files in the reference's column layouts
    def write_cube(self, what: int, field: int, ds: int, directory, name: str, frame: int, time: float) -> None:
        """output_cube: <directory>/<name>-<frame>.raw (FP64, every ds-th site) and the .bov header."""
        _check(_lib.lat_write_cube(self._h, what, field, ds, str(directory).encode(), name.encode(), frame, time))

    def write_energy_line(self, path, time: float) -> None:
        _check(_lib.lat_write_energy_line(self._h, str(path).encode(), time))

    def write_log_line(self, path, time: float) -> None:
        """One LOG.out record of the DEFROST tree (lat_write_log_line)."""
        _check(_lib.lat_write_log_line(self._h, str(path).encode(), time))

    def write_spectrum_block(self, path) -> None:
        _check(_lib.lat_write_spectrum_block(self._h, str(path).encode()))

    # learned closure
    def coarsen(self, nc: int, out: "DeviceArray", offset: int = 0, units: int = 0) -> None:
        """Sharp-k filtered fields, momenta and missing forces on an nc^3 lattice,
        written as FP32 [3 nf][nc^3] at element `offset` of `out`."""
        offset, nc = int(offset), int(nc)
        if offset < 0 or offset + 3 * self.nfld * nc ** 3 > out.size:
            raise ValueError("coarsen output does not fit")
        _check(_lib.lat_coarsen(self._h, nc, units, out.ptr + 4 * offset))

    def attach_closure(self, net: "Net | None", every: int = 1, units: int = 0) -> None:
        _check(_lib.lat_closure_attach(self._h, None if net is None else net._h, every, units))
        self._closure = net  # keeps the network alive while attached



class SlabLattice(Lattice):
    """The z-planes [z0, z1) of a global finite-difference lattice
    (lat_slab_create): one rank's part of a decomposed run.  State arrays
    cover the slab's interior planes, shaped (nfld, z1 - z0, ny, nx).  The
    evolution calls need set_hooks(): a halo exchange filling both ghost
    planes, and an all-reduce of the lattice sums over all slabs."""

    def __init__(self, cfg: LatConfig, z0: int, z1: int):
        lib = load_library()
        self.cfg = cfg
        self._h = C.c_void_p()
        _check(lib.lat_slab_create(C.byref(self._h), C.byref(cfg), int(z0), int(z1)))
        self.nx, self.ny, self.nfld = cfg.nx, cfg.ny, cfg.nfld
        self.nz = int(z1) - int(z0)
        self.z0, self.z1, self.nz_global = int(z0), int(z1), cfg.nz
        self.N = self.nx * self.ny * self.nz
        self._hooks = None
        self.hook_error = None

    def halo_bytes(self) -> int:
        n = C.c_size_t()
        _check(_lib.lat_slab_halo_bytes(self._h, C.byref(n)))
        return n.value

    def halo(self, op: int, dev_ptr: int) -> None:
        """op 0/1: lowest/highest interior plane -> device buffer; 2/3: device buffer -> lower/upper ghost."""
        _check(_lib.lat_slab_halo(self._h, int(op), C.c_void_p(dev_ptr)))

    def set_hooks(self, halo, allreduce) -> None:
        """halo(slab) fills both ghost planes; allreduce(v: np.ndarray) returns
        v summed over all slabs.  An exception in a hook stops the engine call
        with a LatticeError and is kept in ``hook_error``."""
        def _halo(_user, _h):
            try:
                halo(self)
                return 0
            except Exception as e:  # noqa: BLE001
                self.hook_error = e
                return 1

        def _sum(_user, v, n):
            try:
                arr = np.ctypeslib.as_array(v, shape=(n,))
                arr[:] = allreduce(arr.copy())
                return 0
            except Exception as e:  # noqa: BLE001
                self.hook_error = e
                return 1

        self._hooks = (HALO_FN(_halo), SUM_FN(_sum))  # referenced for as long as the handle lives
        _check(_lib.lat_slab_set_hooks(self._h, self._hooks[0], self._hooks[1], None))

class DeviceArray:
    """A flat FP32 device buffer (lat_dev_alloc) for closure data sets."""

    def __init__(self, size: int, device: int = 0):
        load_library()
        self.size = int(size)
        p = C.c_void_p()
        _check(_lib.lat_dev_alloc(device, C.byref(p), 4 * self.size))
        self.ptr = p.value

    def upload(self, a: np.ndarray, offset: int = 0) -> None:
        a = np.ascontiguousarray(a, dtype=np.float32)
        offset = int(offset)
        if offset < 0 or offset + a.size > self.size:
            raise ValueError("upload out of range")
        _check(_lib.lat_memcpy(self.ptr + 4 * offset, a.ctypes.data, 4 * a.size, 0))

    def download(self, count: int | None = None, offset: int = 0) -> np.ndarray:
        offset = int(offset)
        count = self.size - offset if count is None else int(count)
        if offset < 0 or offset + count > self.size:
            raise ValueError("download out of range")
        out = np.empty(count, dtype=np.float32)
        _check(_lib.lat_memcpy(out.ctypes.data, self.ptr + 4 * offset, 4 * count, 1))
        return out

    def close(self) -> None:
        if getattr(self, "ptr", None):
            _lib.lat_dev_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Net:
    """The closure network (lat_net_*): 4 -> 32 -> 32 -> 2 periodic 3^3 convolutions."""

    def __init__(self, device: int = 0, seed: int = 1):
        load_library()
        self._h = C.c_void_p()
        _check(_lib.lat_net_create(C.byref(self._h), device, seed))
        self.nparams = int(_lib.lat_net_nparams())

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _check(_lib.lat_net_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.empty(self.nparams, dtype=np.float32)
        _check(_lib.lat_net_get_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), self.nparams))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(_lib.lat_net_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), p.size))

    def set_norm(self, shift, scale, out_scale) -> None:
        a, b, c = (np.ascontiguousarray(v, dtype=np.float64) for v in (shift, scale, out_scale))
        _check(_lib.lat_net_set_norm(self._h, _dp(a), _dp(b), _dp(c)))

    def norm(self):
        a, b, c = np.zeros(4), np.zeros(4), np.zeros(2)
        _check(_lib.lat_net_get_norm(self._h, _dp(a), _dp(b), _dp(c)))
        return a, b, c

    @staticmethod
    def _idx(idx):
        i = np.ascontiguousarray(idx, dtype=np.int32)
        return i, i.ctypes.data_as(C.POINTER(C.c_int32))

    def forward(self, data: DeviceArray, stride: int, idx, shape) -> np.ndarray:
        i, ip = self._idx(idx)
        nx, ny, nz = (int(v) for v in shape)
        stride = int(stride)
        out = DeviceArray(len(i) * nx * ny * nz * 2)
        _check(_lib.lat_net_forward(self._h, data.ptr, stride, ip, len(i), nx, ny, nz, out.ptr))
        r = out.download().reshape(len(i), nz, ny, nx, 2)
        out.close()
        return r

    def grad(self, data: DeviceArray, stride: int, idx, shape):
        i, ip = self._idx(idx)
        nx, ny, nz = (int(v) for v in shape)
        stride = int(stride)
        loss = C.c_double()
        g = np.empty(self.nparams, dtype=np.float32)
        _check(_lib.lat_net_grad(self._h, data.ptr, stride, ip, len(i), nx, ny, nz, C.byref(loss),
                                 g.ctypes.data_as(C.POINTER(C.c_float))))
        return loss.value, g

    def train_step(self, data: DeviceArray, stride: int, idx, shape, lr: float) -> float:
        i, ip = self._idx(idx)
        nx, ny, nz = (int(v) for v in shape)
        stride = int(stride)
        loss = C.c_double()
        _check(_lib.lat_net_train_step(self._h, data.ptr, stride, ip, len(i), nx, ny, nz, lr, C.byref(loss)))
        return loss.value

    def launch_count(self) -> int:
        return int(_lib.lat_net_launch_count(self._h))

    def time_forward(self, shape, reps: int = 10) -> np.ndarray:
        """ms of (input packing, conv1, conv2, conv3) on an nx x ny x nz lattice."""
        nx, ny, nz = (int(v) for v in shape)
        ms = np.zeros(4)
        _check(_lib.lat_net_time_forward(self._h, nx, ny, nz, reps, _dp(ms)))
        return ms


class Ensemble:
    """A batch of independent spectral runs of uneven sizes advanced together."""

    def __init__(self, cfg: LatConfig, sizes):
        lib = load_library()
        self.sizes = [int(s) for s in sizes]
        arr = (C.c_int32 * len(self.sizes))(*self.sizes)
        self._h = C.c_void_p()
        self.cfg = cfg
        _check(lib.lat_ens_create(C.byref(self._h), C.byref(cfg), len(self.sizes), arr))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.lat_ens_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init_vacuum(self, seeds, fld0, dfld0, m2eff, amp=1e-8, kcut_frac=0.5):
        s = (C.c_uint64 * len(seeds))(*[int(x) for x in seeds])
        _check(_lib.lat_ens_init_vacuum(self._h, s, fld0, dfld0, m2eff, amp, kcut_frac))

    def symp(self, order, dt_over_dx, nsteps):
        _check(_lib.lat_ens_symp(self._h, order, dt_over_dx, nsteps))

    def sync(self):
        _check(_lib.lat_ens_sync(self._h))

    def prepare_symp(self, order, dt_over_dx, nsteps):
        _check(_lib.lat_ens_prepare(self._h, order, dt_over_dx, nsteps))

    def mark(self, slot):
        _check(_lib.lat_ens_mark(self._h, slot))

    def mark_elapsed(self, a, b) -> float:
        ms = C.c_double()
        _check(_lib.lat_ens_mark_elapsed(self._h, a, b, C.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        n = C.c_int64()
        _check(_lib.lat_ens_launch_count(self._h, C.byref(n)))
        return n.value

    def autotune(self, cache_path=None):
        _check(_lib.lat_ens_autotune(self._h, None if cache_path is None else str(cache_path).encode()))

    def tuning(self):
        out = (C.c_int32 * 2)()
        _check(_lib.lat_ens_tuning_get(self._h, out))
        return list(out)

    def sep_streamed(self) -> bool:
        on = C.c_int32()
        _check(_lib.lat_ens_sep_streamed(self._h, C.byref(on)))
        return bool(on.value)

    def energies(self):
        out = np.zeros((len(self.sizes), NENERGY))
        _check(_lib.lat_ens_energies(self._h, _dp(out)))
        return out

    def spectrum(self, run, nbins):
        S, W = np.zeros(nbins), np.zeros(nbins)
        _check(_lib.lat_ens_spectrum(self._h, run, nbins, _dp(S), _dp(W)))
        return S, W

    def state(self, run):
        n = self.sizes[run]
        f = np.empty((n, n, n))
        p = np.empty_like(f)
        _check(_lib.lat_ens_download(self._h, run, _dp(f), _dp(p)))
        return f, p


def laplacian_3d(f: np.ndarray, dk: float) -> np.ndarray:
    """laplacian_3d(n1,n2,n3,f,Fk,dk,planf,planb) on a (n3,n2,n1) C-order array."""
    load_library()
    g = np.ascontiguousarray(f, np.float64).copy()
    n3, n2, n1 = g.shape
    _check(_lib.lat_laplacian_3d(n1, n2, n3, _dp(g), dk))
    return g


def spectrum_3d(f: np.ndarray, mode=SPEC_WEIGHTED, nbins=None):
    load_library()
    g = np.ascontiguousarray(f, np.float64)
    n3, n2, n1 = g.shape
    if nbins is None:
        nbins = int(np.floor(np.sqrt((n1 // 2 + 1) ** 2 + (n2 // 2 + 1) ** 2 + (n3 // 2 + 1) ** 2 + 1.0)))
    S, W = np.zeros(nbins), np.zeros(nbins)
    _check(_lib.lat_spectrum_3d(n1, n2, n3, _dp(g), mode, nbins, _dp(S), _dp(W)))
    return S, W


def host_alloc(nbytes: int) -> int:
    load_library()
    p = C.c_void_p()
    _check(_lib.lat_host_alloc(C.byref(p), nbytes))
    return p.value


def host_free(ptr: int) -> None:
    _lib.lat_host_free(C.c_void_p(ptr))
