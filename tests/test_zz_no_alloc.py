"""The allocation-free spectrum entry point against the regular one.

lat_spectrum_noalloc serves callers that cannot call cudaMalloc (a driver that
owns the whole device through its own memory pool, or a time loop that must
not allocate): it takes a half spectrum and an output buffer already on the
device and keeps its scratch in a fixed static device array.  This test gives
it the half spectrum of a lattice field (made here with torch, since the test
itself may allocate), calls it twice in a row, and checks both results against
lat_spectrum on the same field; around the second call the device's free
memory must not change (a cudaMalloc, or a library routine that allocates a
workspace, would show up there).  It lives in its own file, collected last, so
that a run stopping at the first failure has already run every other test
when this one fails; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(engine, F, shape, prec, mode, nbins, out, torch):
    nz, ny, nx = shape
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = engine._lib.lat_spectrum_noalloc(ctypes.c_void_p(F.data_ptr()), nx, ny, nz, prec, mode, nbins,
                                          ctypes.c_void_p(out.data_ptr()), stream)
    assert rc == 0, engine._lib.lat_last_error().decode()
    torch.cuda.synchronize()
    return out[:nbins].cpu().numpy().copy(), out[nbins:].cpu().numpy().copy()


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 1e-5)])
@pytest.mark.parametrize("mode", [0, 1])
def test_spectrum_noalloc_matches_lat_spectrum(engine, prec, tol, mode):
    torch = pytest.importorskip("torch")
    shape = (16, 24, 32)  # (nz, ny, nx)
    cfg = engine.make_config((shape[2], shape[1], shape[0]), nfld=1, length=8.0, precision=prec)
    g = engine.Lattice(cfg)
    rng = np.random.default_rng(17)
    f = 1.0 + 0.1 * rng.standard_normal(shape)
    g.set_state(f[None], np.zeros((1,) + shape))
    nbins = g.nbins()
    S_ref, W_ref = g.spectrum(engine.SPEC_FLD, 0, mode, nbins)
    dtype = torch.float64 if prec == 0 else torch.float32
    stored = f if prec == 0 else f.astype(np.float32)  # the FP32 lattice transforms its FP32 field
    F = torch.fft.rfftn(torch.from_numpy(np.ascontiguousarray(stored)).to("cuda", dtype)).contiguous()
    out = torch.full((2 * nbins,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):  # two calls in a row share the static scratch
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        S, W = _noalloc(engine, F, shape, prec, mode, nbins, out, torch)
        if call == 1:  # the first call may load the module's device code; the second allocates nothing
            assert torch.cuda.mem_get_info()[0] == free0
        assert np.max(np.abs(S - S_ref)) <= tol * np.max(np.abs(S_ref))
        if mode == 1:
            assert np.array_equal(W, W_ref)
        else:
            assert np.max(np.abs(W - W_ref)) <= 1e-12 * np.max(W_ref)


def test_spectrum_noalloc_rejects_oversize(engine):
    torch = pytest.importorskip("torch")
    F = torch.zeros((4, 4, 3), dtype=torch.complex128, device="cuda")
    out = torch.zeros(2 * 600, dtype=torch.float64, device="cuda")
    rc = engine._lib.lat_spectrum_noalloc(ctypes.c_void_p(F.data_ptr()), 4, 4, 4, 0, 0, 600,
                                          ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 1
    assert b"512" in engine._lib.lat_last_error()
