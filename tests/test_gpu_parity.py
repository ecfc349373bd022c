"""GPU engine vs CPU oracle on identical inputs (FP64: <= 1e-10 relative).

Every evolution test starts both sides from the same state, runs the same
reference call sequence (symp / o2step / Hamiltonian_Split) and compares the
fields, momenta and Friedmann scalars.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import rel_err
from helpers import L, bubble_fd27, cfg, phi4_fd7, two_field_spectral, random_state, vacuum_ic

pytestmark = pytest.mark.gpu
TOL64 = 1e-10


def pair(engine, orc, c):
    return engine.Lattice(c), orc.Oracle(c)


def same_start(g, o, seed=1, mean=1.0, amp=0.05):
    f, p = random_state((g.nfld, g.nz, g.ny, g.nx), seed=seed, mean=mean, amp=amp)
    g.set_state(f, p)
    o.set_state(f, p)
    return f, p


def compare_state(g, o, tol=TOL64):
    gf, gp = g.get_state()
    of, op = o.get_state()
    assert rel_err(gf, of) <= tol, rel_err(gf, of)
    assert rel_err(gp, op) <= tol, rel_err(gp, op)


@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_fd7_minkowski_symp(engine, orc, order):
    c = phi4_fd7(16)
    g, o = pair(engine, orc, c)
    same_start(g, o)
    dt = c.len / c.nx / 10
    g.symp(order, dt, 5)
    o.symp(order, dt, 5)
    compare_state(g, o)
    assert np.allclose(g.time(), o.time(), rtol=0, atol=1e-15)


def test_fd7_64cube_100_steps(engine, orc):
    """The 64^3 plain-method workload (L=20, dt=dx/10, phi^4, FD7, leapfrog), 100 steps."""
    c = phi4_fd7(64)
    g, o = pair(engine, orc, c)
    vacuum_ic(g, seed=1000, amp=1e-8)
    vacuum_ic(o, seed=1000, amp=1e-8)
    compare_state(g, o, 1e-12)
    dt = (20.0 / 64) / 10
    for _ in range(10):
        g.symp(2, dt, 10)
        o.symp(2, dt, 10)
    compare_state(g, o)
    eg, eo = g.energies(), o.energies()
    assert abs(eg[L.E_RHO] - eo[L.E_RHO]) <= 1e-10 * abs(eo[L.E_RHO])


@pytest.mark.parametrize("split", [L.SPLIT_PSEUDOSPEC, L.SPLIT_DEFROST])
def test_fd27_gw_minkowski(engine, orc, split):
    c = bubble_fd27(16, split=split)
    g, o = pair(engine, orc, c)
    same_start(g, o, mean=0.0, amp=0.3)
    dt = 0.25 / 10
    g.symp(2, dt, 12)
    o.symp(2, dt, 12)
    compare_state(g, o)
    gu, gpu_ = g.gw_state()
    ou, opu = o.gw_state()
    assert rel_err(gu, ou) <= TOL64
    assert rel_err(gpu_, opu) <= TOL64
    Sg, Wg = g.gw_spectrum(16)
    So, Wo = o.gw_spectrum(16)
    assert np.array_equal(Wg, Wo)
    assert rel_err(Sg, So) <= 1e-9


@pytest.mark.parametrize("shape", [(32, 16, 12), (64, 8, 8), (48, 8, 8)])
def test_fd_fp32_tile_rows(engine, orc, shape):
    """FP32-Kahan stencil passes against the FP64 oracle.  Rows of 32 and 64
    sites are whole tiles (staged by 16-byte copies into padded rows); 48 has
    a partial tile (4-byte copies).  FD27 with GW sourcing and FD7."""
    nx, ny, nz = shape
    for lap, gw in ((L.LAP_FD27, True), (L.LAP_FD7, False)):
        c = L.make_config(shape, nfld=1, length=0.25 * nx, laplacian=lap, background=L.BG_MINKOWSKI,
                          precision=L.FP32_KAHAN, model=L.MODEL_DOUBLE_WELL, model_params=(0.01,), gw=gw,
                          gw_coupling=2.0)
        g, o = pair(engine, orc, c)
        same_start(g, o, mean=0.0, amp=0.3)
        dt = 0.25 / 10
        g.symp(2, dt, 12)
        o.symp(2, dt, 12)
        compare_state(g, o, 5e-6)
        if gw:
            gu, gpu_ = g.gw_state()
            ou, opu = o.gw_state()
            assert rel_err(gu, ou) <= 1e-4, rel_err(gu, ou)
            assert rel_err(gpu_, opu) <= 1e-4, rel_err(gpu_, opu)
        g.close()


def test_fd27_conformal_plain_path(engine, orc):
    c = L.make_config(16, nfld=2, length=8.0, laplacian=L.LAP_FD27, background=L.BG_CONFORMAL,
                      model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    g, o = pair(engine, orc, c)
    same_start(g, o)
    g.calc_metric()
    o.calc_metric()
    assert abs(g.scale_factor()[1] - o.scale_factor()[1]) <= 1e-12 * abs(o.scale_factor()[1])
    g.symp(4, 0.05, 6)
    o.symp(4, 0.05, 6)
    compare_state(g, o)
    (ag, apg), (ao, apo) = g.scale_factor(), o.scale_factor()
    assert abs(ag - ao) <= 1e-12 * ao and abs(apg - apo) <= 1e-10 * abs(apo)


@pytest.mark.parametrize("conformal", [False, True])
def test_spectral_two_field_fused(engine, orc, conformal):
    c = two_field_spectral(32, conformal=conformal)
    g, o = pair(engine, orc, c)
    vacuum_ic(g, amp=1e-3)
    vacuum_ic(o, amp=1e-3)
    if conformal:
        g.calc_metric()
        o.calc_metric()
    dt = c.len / c.nx / 20
    for _ in range(4):
        g.symp(4, dt, 5)
        o.symp(4, dt, 5)
    compare_state(g, o)
    if conformal:
        (ag, apg), (ao, apo) = g.scale_factor(), o.scale_factor()
        assert abs(ag - ao) <= 1e-12 * ao
        assert abs(apg - apo) <= 1e-10 * abs(apo)


def test_spectral_o2step_and_split(engine, orc):
    c = two_field_spectral(16, conformal=True)
    g, o = pair(engine, orc, c)
    same_start(g, o, amp=0.02)
    for obj in (g, o):
        obj.set_scale_factor(1.0, -0.5)
        obj.hamiltonian_split(0.01, 1)
        obj.o2step(0.02, 0.6, 0.4)
        obj.hamiltonian_split(0.03, 3)
        obj.hamiltonian_split(0.01, 2)
    compare_state(g, o)
    assert np.allclose(g.scale_factor(), o.scale_factor(), rtol=1e-12, atol=0)
    assert np.allclose(g.time(), o.time(), rtol=0, atol=1e-15)


def test_laplacians(engine, orc):
    for c in (two_field_spectral(16, conformal=False), phi4_fd7(16),
              L.make_config((16, 12, 10), nfld=1, length=5.0, laplacian=L.LAP_FD27)):
        g, o = pair(engine, orc, c)
        same_start(g, o)
        assert rel_err(g.laplacian(0), o.laplacian(0)) <= 1e-12


def test_standalone_laplacian_3d(engine):
    n1, n2, n3 = 16, 12, 8
    dk = 0.7
    x = np.arange(n1)[None, None, :]
    y = np.arange(n2)[None, :, None]
    f = np.cos(2 * np.pi * 3 * x / n1) * np.sin(2 * np.pi * 2 * y / n2) + 0 * np.zeros((n3, 1, 1))
    lap = engine.laplacian_3d(f, dk)
    expect = -((3 * dk) ** 2 + (2 * dk) ** 2) * f
    assert np.max(np.abs(lap - expect)) <= 1e-12 * np.max(np.abs(expect))


def test_vacuum_ic_identical(engine, orc):
    c = two_field_spectral(32)
    g, o = pair(engine, orc, c)
    vacuum_ic(g, seed=1001, amp=1e-8)
    vacuum_ic(o, seed=1001, amp=1e-8)
    compare_state(g, o, 1e-12)


@pytest.mark.parametrize("n,prec", [(16, L.FP64), (32, L.FP64), (32, L.FP32_KAHAN)])
def test_sample_ic_matches_oracle(engine, orc, n, prec):
    """The reference's sample() generator (DST-II of the oversampled radial
    profile through a length-4 nos FFT, noise per mode) against the oracle,
    whose DST is the direct sum; fluctuations compared relative to their size."""
    c = two_field_spectral(n, prec)
    g, o = pair(engine, orc, c)
    fld0, dfld0 = [1.0, 0.25], [0.1, -0.2]
    g.init_sample(77, fld0, dfld0, 3.0, mpl=0.5)
    o.init_sample(77, fld0, dfld0, 3.0, mpl=0.5)
    gf, gp = g.get_state()
    of, op = o.get_state()
    tol = 1e-10 if prec == L.FP64 else 1e-6
    for l in range(2):
        df, dp_ = of[l] - fld0[l], op[l] - dfld0[l]
        assert np.max(np.abs(gf[l] - of[l])) <= tol * np.max(np.abs(df)) + 1e-15
        assert np.max(np.abs(gp[l] - op[l])) <= tol * np.max(np.abs(dp_)) + 1e-15
        assert np.std(df) > 0 and np.std(dp_) > 0
    if n == 16:  # cubic lattices only
        nc = L.make_config((16, 16, 8), nfld=2, length=4.0, laplacian=L.LAP_SPECTRAL)
        h = engine.Lattice(nc)
        with pytest.raises(engine.LatticeError):
            h.init_sample(1, [0, 0], [0, 0], 1.0)
        h.close()


def test_energies(engine, orc):
    for c in (phi4_fd7(16), bubble_fd27(12), two_field_spectral(16, conformal=True)):
        g, o = pair(engine, orc, c)
        same_start(g, o)
        if c.background == L.BG_CONFORMAL:
            g.set_scale_factor(1.3, -0.7)
            o.set_scale_factor(1.3, -0.7)
        eg, eo = g.energies(), o.energies()
        for i in range(L.NENERGY):
            assert abs(eg[i] - eo[i]) <= 1e-10 * max(abs(eo[i]), 1e-300), (i, eg[i], eo[i])
        assert abs(eg[L.E_GE_LAP] - eg[L.E_GE_GRAD]) <= 1e-10 * abs(eg[L.E_GE_LAP])


def test_spectra_modes_exact(engine, orc):
    c = two_field_spectral(24, conformal=False)
    g, o = pair(engine, orc, c)
    same_start(g, o)
    for what in (L.SPEC_FLD, L.SPEC_FLDP):
        for mode in (L.SPEC_WEIGHTED, L.SPEC_COUNT):
            Sg, Wg = g.spectrum(what, 1, mode)
            So, Wo = o.spectrum(what, 1, mode)
            if mode == L.SPEC_COUNT:
                assert np.array_equal(Wg, Wo)  # bit-exact integer mode counts
            else:
                assert rel_err(Wg, Wo) <= 1e-13
            assert rel_err(Sg, So) <= 1e-11
    Srg, Sig = g.crossspec_3d(L.SPEC_FLD, 0, L.SPEC_FLDP, 1)
    Sro, Sio = o.crossspec_3d(L.SPEC_FLD, 0, L.SPEC_FLDP, 1)
    assert rel_err(Srg, Sro) <= 1e-11 and rel_err(Sig, Sio) <= 1e-11


def test_standalone_spectrum_3d(engine, orc):
    rng = np.random.default_rng(3)
    f = rng.standard_normal((10, 12, 16))
    c = L.make_config((16, 12, 10), nfld=1, length=1.0)
    o = orc.Oracle(c)
    o.set_state(f[None])
    for mode in (L.SPEC_WEIGHTED, L.SPEC_COUNT):
        Sg, Wg = engine.spectrum_3d(f, mode)
        So, Wo = o.spectrum(0, 0, mode)
        assert rel_err(Sg, So) <= 1e-12
        if mode == L.SPEC_COUNT:
            assert np.array_equal(Wg, Wo)


def test_bubbles_ic(engine, orc):
    c = bubble_fd27(32, gw=False)
    g, o = pair(engine, orc, c)
    cen = [[4.0, 4.0, 4.0], [4.0 + 2.5, 4.0, 4.0]]
    g.init_bubbles(cen, 1.5, math.sqrt(2))
    o.init_bubbles(cen, 1.5, math.sqrt(2))
    compare_state(g, o, 1e-13)


def test_fortran_layout_padding(engine):
    c = phi4_fd7(8)
    c.nfld = 2
    c.model = L.MODEL_PHI4_G2
    g = engine.Lattice(c)
    n = 8
    rng = np.random.default_rng(5)
    # DEFROST padding: 2 low, 3 high ghost sites per side (latpar.f90:78-80)
    lo, hi = 2, 3
    m = n + lo + hi
    fld = rng.standard_normal((m, m, m, 2))
    fldp = rng.standard_normal((n, n, n, 2))
    g.upload_fortran(fld, lo, hi, fldp, 0, 0)
    f, p = g.get_state()
    inner = fld[lo:lo + n, lo:lo + n, lo:lo + n, :]
    assert np.array_equal(f, np.moveaxis(inner, -1, 0))
    assert np.array_equal(p, np.moveaxis(fldp, -1, 0))
    back = np.full_like(fld, -7.0)
    backp = np.zeros_like(fldp)
    g.download_fortran(back, lo, hi, backp, 0, 0)
    assert np.array_equal(back[lo:lo + n, lo:lo + n, lo:lo + n, :], inner)
    mask = np.ones(back.shape, bool)
    mask[lo:lo + n, lo:lo + n, lo:lo + n, :] = False
    assert np.all(back[mask] == -7.0)  # ghost sites untouched


@pytest.mark.parametrize("prec", [L.FP64, L.FP32_KAHAN])
def test_pinned_host_arrays_direct(engine, prec):
    """Unpadded pinned arrays are converted in place over the CPU-GPU link;
    the result must equal the staged copy of the same pageable arrays."""
    import ctypes

    c = phi4_fd7(16, prec)
    c.nfld = 2
    c.model = L.MODEL_PHI4_G2
    n, nf = 16, 2
    rng = np.random.default_rng(11)
    fld = rng.standard_normal((n, n, n, nf))
    fldp = rng.standard_normal((n, n, n, nf))
    nbytes = fld.nbytes
    ptrs = [engine.host_alloc(nbytes) for _ in range(2)]
    try:
        pin = [np.ctypeslib.as_array((ctypes.c_double * fld.size).from_address(p)).reshape(fld.shape) for p in ptrs]
        pin[0][...] = fld
        pin[1][...] = fldp
        a, b = engine.Lattice(c), engine.Lattice(c)
        a.upload_fortran(pin[0], 0, 0, pin[1], 0, 0)
        b.upload_fortran(fld, 0, 0, fldp, 0, 0)
        fa, pa = a.get_state()
        fb, pb = b.get_state()
        assert np.array_equal(fa, fb) and np.array_equal(pa, pb)
        for g in (a, b):
            g.symp(2, 0.05, 3)
        pin[0][...] = -1.0
        pin[1][...] = -1.0
        a.download_fortran(pin[0], 0, 0, pin[1], 0, 0)
        back, backp = np.empty_like(fld), np.empty_like(fldp)
        b.download_fortran(back, 0, 0, backp, 0, 0)
        assert np.array_equal(pin[0], back) and np.array_equal(pin[1], backp)
        a.close()
        b.close()
    finally:
        for p in ptrs:
            engine.host_free(p)


@pytest.mark.parametrize("prec", [L.FP64, L.FP32_KAHAN])
@pytest.mark.parametrize("nf", [1, 2])
@pytest.mark.parametrize("shape", [(12, 8, 16), (7, 5, 3)])
def test_layout_conversion_exact(engine, prec, nf, shape):
    """FP64 host arrays <-> device state, bit for bit: FP64 kept as is; FP32
    fields as hi = fl32(v), c = fl32(hi - v), read back as hi - c; FP32 momenta
    as fl32(v), on an even and an odd site count."""
    nx, ny, nz = shape
    c = cfg((nx, ny, nz), nfld=nf, length=4.0, laplacian=L.LAP_FD7, background=L.BG_MINKOWSKI, precision=prec,
            model=L.MODEL_PHI4 if nf == 1 else L.MODEL_PHI4_G2, model_params=(1.0,) if nf == 1 else (1.0, 2.0))
    g = engine.Lattice(c)
    rng = np.random.default_rng(17)
    f = rng.standard_normal((nf, nz, ny, nx)) * np.exp(rng.uniform(-20, 20, (nf, nz, ny, nx)))
    p = rng.standard_normal((nf, nz, ny, nx))
    g.set_state(f, p)
    fb, pb = g.get_state()
    g.close()
    if prec == L.FP64:
        assert np.array_equal(fb, f) and np.array_equal(pb, p)
        return
    hi = f.astype(np.float32)
    cc = (hi.astype(np.float64) - f).astype(np.float32)
    assert np.array_equal(fb, hi.astype(np.float64) - cc.astype(np.float64))
    assert np.array_equal(pb, p.astype(np.float32).astype(np.float64))


def test_checkpoint_roundtrip(engine, tmp_path):
    c = two_field_spectral(16, conformal=True)
    g = engine.Lattice(c)
    vacuum_ic(g, amp=1e-3)
    g.set_scale_factor(1.25, -0.75)
    g.checkpoint_write(tmp_path, 3.5, 7)
    f, p = g.get_state()
    h = engine.Lattice(c)
    t, fr = h.checkpoint_read(tmp_path)
    assert (t, fr) == (3.5, 7)
    f2, p2 = h.get_state()
    assert np.array_equal(f, f2) and np.array_equal(p, p2)
    assert h.scale_factor() == (1.25, -0.75)
    raw = np.fromfile(tmp_path / "fld_2.raw")
    assert np.array_equal(raw.reshape(16, 16, 16), f[1])


def test_checkpoint_corrupt_header(engine, tmp_path):
    c = phi4_fd7(8)
    g = engine.Lattice(c)
    g.checkpoint_write(tmp_path)
    (tmp_path / "checkpt.dat").write_text("garbage\n")
    with pytest.raises(engine.LatticeError) as e:
        g.checkpoint_read(tmp_path)
    assert e.value.code == 7
    (tmp_path / "fld_1.raw").write_bytes(b"\0" * 100)
    with pytest.raises(engine.LatticeError):
        g.checkpoint_read(tmp_path)


def test_deterministic_reductions(engine):
    c = two_field_spectral(32, conformal=True)
    outs = []
    for _ in range(2):
        g = engine.Lattice(c)
        vacuum_ic(g, amp=1e-3)
        g.calc_metric()
        g.symp(4, 0.01, 10)
        outs.append((g.get_state(), g.scale_factor()))
    (f1, p1), s1 = outs[0]
    (f2, p2), s2 = outs[1]
    assert np.array_equal(f1, f2) and np.array_equal(p1, p2) and s1 == s2


def test_graph_replay_matches_eager(engine, monkeypatch):
    c = phi4_fd7(16)
    g = engine.Lattice(c)
    f, p = random_state((1, 16, 16, 16), seed=9)
    g.set_state(f, p)
    for _ in range(3):
        g.symp(2, 0.03, 3)  # first call captures a graph, later calls replay it
    a = g.get_state()
    g.timing(True)  # timing disables graphs: eager launches
    g.set_state(f, p)
    for _ in range(3):
        g.symp(2, 0.03, 3)
    b = g.get_state()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_prepared_graph_leaves_state_and_replays(engine):
    """lat_symp_prepare captures without running: state, scale factor and time
    are unchanged, and the next symp call replays the prepared graph."""
    c = L.make_config((64, 32, 32), nfld=2, length=16.0, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                      precision=L.FP32_KAHAN, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0),
                      spectral_impl=L.SPEC_IMPL_SEPARABLE)
    f, p = random_state((2, 32, 32, 64), seed=12)
    out = []
    for prepare in (False, True):
        g = engine.Lattice(c)
        g.set_state(f, p)
        g.set_scale_factor(1.0, 0.0)
        g.calc_metric()
        before = g.get_state(), g.scale_factor(), g.time()
        if prepare:
            g.prepare_symp(4, 0.01, 3)
            assert np.array_equal(g.get_state()[0], before[0][0])
            assert g.scale_factor() == before[1] and list(g.time()) == list(before[2])
            l0 = g.launch_count()
        g.symp(4, 0.01, 3)
        if prepare:
            assert g.launch_count() > l0
        out.append((g.get_state(), g.scale_factor()))
        g.close()
    assert np.array_equal(out[0][0][0], out[1][0][0]) and np.array_equal(out[0][0][1], out[1][0][1])
    assert out[0][1] == out[1][1]


@pytest.mark.parametrize("prec", [L.FP64, L.FP32_KAHAN])
def test_output_cube_bov(engine, tmp_path, prec):
    """output_cube's brick of values: every ds-th site as FP64, x fastest,
    and the .bov header VisIt reads (outputfile.f90:942-1016)."""
    c = L.make_config((16, 8, 12), nfld=2, length=8.0, laplacian=L.LAP_FD27, precision=prec,
                      model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    g = engine.Lattice(c)
    f, p = random_state((2, 12, 8, 16), seed=41, mean=0.3, amp=0.1)
    g.set_state(f, p)
    gf, gp = g.get_state()
    for what, field, ds, arr in ((L.SPEC_FLD, 1, 2, gf), (L.SPEC_FLDP, 0, 4, gp), (L.SPEC_FLD, 0, 1, gf)):
        g.write_cube(what, field, ds, tmp_path, "fld", 7 + ds, 1.25)
        raw = np.fromfile(tmp_path / f"fld-{7 + ds:05d}.raw", dtype="<f8")
        want = arr[field][::ds, ::ds, ::ds]
        assert raw.size == want.size and np.array_equal(raw.reshape(want.shape), want)
        hdr = dict(ln.split(":", 1) for ln in (tmp_path / f"fld-{7 + ds:05d}.bov").read_text().splitlines())
        assert float(hdr["TIME"]) == 1.25 and hdr["VARIABLE"].strip() == "fld"
        assert [float(x) for x in hdr["BRICK_SIZE"].split()] == [8.0, 4.0, 6.0]
        assert [int(x) for x in hdr["DATA_SIZE"].split()] == [16 // ds, 8 // ds, 12 // ds]
        assert hdr["DATA_FILE"].strip() == f"fld-{7 + ds:05d}.raw"
        assert hdr["DATA_FORMAT"].strip() == "DOUBLE" and hdr["CENTERING"].strip() == "zonal"
    with pytest.raises(engine.LatticeError):
        g.write_cube(L.SPEC_FLD, 0, 3, tmp_path, "fld", 1, 0.0)  # 16 is not a multiple of 3


def test_log_out_record(engine, orc, tmp_path):
    """LOG.out of the DEFROST tree (output_log_file, iofile.f90:614-630): t, a,
    H, <rho>, rhoball, KE, PE, GE, GE(lap), -3H^2, hamiltonian, with rhoball
    summed over the sites within sqrt(45) of the grid centre."""
    c = L.make_config(32, nfld=2, length=32.0, laplacian=L.LAP_FD27, background=L.BG_CONFORMAL,
                      model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    g, o = pair(engine, orc, c)
    same_start(g, o, mean=0.5, amp=0.2)
    for obj in (g, o):
        obj.set_scale_factor(1.3, -0.7)
    path = tmp_path / "LOG.out"
    g.write_log_line(path, 2.5)
    g.write_log_line(path, 2.5)
    lines = path.read_text().splitlines()
    assert lines[0].startswith("#") and len(lines) == 3
    rows = [np.array([float(v) for v in ln.split()]) for ln in lines[1:]]
    assert np.array_equal(rows[0], rows[1]) and rows[0].size == 11
    e = o.energies()
    a, ap = 1.3, -0.7
    H = -ap / 6.0 / a ** 2
    T, G, V = o.rho_ball_sums(45.0)
    dx = 1.0
    cc = 30.0  # the 27-point stencil's normalisation
    rhoball = 0.5 / a ** 6 * T + 0.25 / (a * dx) ** 2 / cc * G + V
    ke, pe, ge, gel = e[L.E_KE], e[L.E_PE], e[L.E_GE_GRAD], e[L.E_GE_LAP]
    want = [2.5, a, H, ke + ge + pe, rhoball, ke, pe, ge, gel, -3 * H * H, ge + ke + pe - 3 * H * H]
    assert 0 < T and 0 < G
    for i, (got, w) in enumerate(zip(rows[0], want)):
        assert abs(got - w) <= 1e-10 * max(abs(w), 1e-300), (i, got, w)
    spec = engine.Lattice(two_field_spectral(16))
    with pytest.raises(engine.LatticeError):
        spec.write_log_line(tmp_path / "x.out", 0.0)
    spec.close()


def test_output_files_reference_layout(engine, tmp_path):
    """energy_spec.out and spectrum.out records in the reference's column
    layout (ES22.15 + 2X fields), with the values of the engine's reductions."""
    n = 16
    c = L.make_config(n, nfld=2, length=8.0, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                      model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    g = engine.Lattice(c)
    f, p = random_state((2, n, n, n), seed=31, mean=0.7, amp=0.1)
    g.set_state(f, p)
    g.set_scale_factor(1.0, 0.0)
    g.calc_metric()
    ef, sf = tmp_path / "energy_spec.out", tmp_path / "spectrum.out"
    g.write_energy_line(ef, 0.0)
    g.symp(4, 0.02, 3)
    g.write_energy_line(ef, 0.06)
    g.write_spectrum_block(sf)
    lines = ef.read_text().splitlines()
    assert len(lines) == 2
    for ln in lines:
        assert len(ln) == 11 * 24
        assert all(ln[24 * i + 22:24 * i + 24] == "  " for i in range(11))
    row = np.array([float(ln[24 * i:24 * i + 22]) for i in range(11) for ln in lines[1:]])
    e = g.energies()
    a, ap = g.scale_factor()
    ref = [0.06, a, e[L.E_RHO], e[L.E_KE], e[L.E_PE], e[L.E_GE_LAP], e[L.E_GRAV],
           (e[L.E_RHO] + e[L.E_GRAV]) / e[L.E_RHO], -ap * ap / 12 / a ** 4, e[L.E_MEAN0], e[L.E_MEAN1]]
    assert np.allclose(row, ref, rtol=1e-14, atol=1e-300)
    assert abs(row[6] - row[8]) <= 1e-12 * abs(row[6])  # -3H^2 printed twice, two formulas
    blk = sf.read_text().split("\n")
    ns = g.nbins()
    assert blk[ns] == "" and len(blk[0]) == 7 * 24
    tab = np.array([[float(ln[24 * i:24 * i + 22]) for i in range(7)] for ln in blk[:ns]])
    S1, _ = g.spectrum(L.SPEC_FLD, 0, L.SPEC_WEIGHTED, ns)
    S2, _ = g.spectrum(L.SPEC_FLDP, 0, L.SPEC_WEIGHTED, ns)
    Cr, Ci = g.crossspec_3d(L.SPEC_FLDP, 0, L.SPEC_FLD, 0, ns)
    assert np.allclose(tab[:, 0], np.arange(ns) * 2 * math.pi / 8.0, rtol=1e-15)
    for col, ref in ((1, S1), (2, S2), (3, Cr), (4, Ci)):
        assert np.allclose(tab[:, col], ref, rtol=1e-14, atol=0), col
    assert np.all(tab[:, 5:] == 0)


def test_boosted_bubbles_match_restatement(engine):
    """lat_init_bubbles_boosted against a numpy restatement of
    ic_bubble.f90 init_fields/initbubble with the init_cond.f90 profile,
    centres at the reference's getbubpos positions (n/2 +- n/5)."""
    n, dx = 32, 0.25
    c = L.make_config(n, nfld=1, length=n * dx, laplacian=L.LAP_FD27, model=L.MODEL_DOUBLE_WELL,
                      model_params=(0.01,), split_order=L.SPLIT_DEFROST)
    g = engine.Lattice(c)
    cen = [[n // 2 + n // 5, n // 2, n // 2], [n // 2 - n // 5, n // 2, n // 2]]
    r0, pf, pt = 2.0, -1.0, 1.0
    t0 = 1.3 * r0
    g.init_bubbles_boosted(cen, r0, t0, pf, pt)
    f, p = g.get_state()
    i = np.arange(1, n + 1)
    K, J, I = np.meshgrid(i, i, i, indexing="ij")
    step, ave = (pf - pt) / 2, (-pf + pt) / 2
    ef = np.zeros((n, n, n))
    ep = np.zeros((n, n, n))
    for cx, cy, cz in cen:
        rad = np.sqrt(((I - cx) ** 2 + (J - cy) ** 2 + (K - cz) ** 2) * dx * dx)
        out = rad ** 2 > t0 ** 2
        s1 = np.sqrt(np.where(out, rad ** 2 - t0 ** 2, 1.0))
        s = s1 - r0
        ef += np.where(out, step * np.tanh(s / np.sqrt(2)) + ave, pt - pf)
        ep += np.where(out, -step * t0 / s1 / np.sqrt(2) / np.cosh(s / np.sqrt(2)) ** 2, 0.0)
    ef += pf
    assert np.max(np.abs(f[0] - ef)) <= 1e-13
    assert np.max(np.abs(p[0] - ep)) <= 1e-13
    assert np.max(np.abs(ep)) > 0.1  # the walls move


@pytest.mark.parametrize("lap", [L.LAP_FD7, L.LAP_FD27, L.LAP_SPECTRAL])
def test_non_cubic_lattices(engine, orc, lap):
    """Uneven sides, one of them not a power of two (24: radix 3 in both FFTs)."""
    shape = (32, 24, 16)
    c = L.make_config(shape, nfld=2, length=12.0, laplacian=lap, background=L.BG_CONFORMAL,
                      model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    g, o = pair(engine, orc, c)
    same_start(g, o, amp=0.05)
    for obj in (g, o):
        obj.set_scale_factor(1.0, 0.0)
        obj.calc_metric()
        obj.symp(4, 0.02, 6)
    compare_state(g, o)
    assert np.allclose(g.scale_factor(), o.scale_factor(), rtol=1e-11, atol=0)
    nb = 20
    Sg, Wg = g.spectrum(L.SPEC_FLD, 1, L.SPEC_COUNT, nb)
    So, Wo = o.spectrum(L.SPEC_FLD, 1, L.SPEC_COUNT, nb)
    assert np.array_equal(Wg, Wo)
    assert rel_err(Sg, So) <= 1e-10


def test_spectral_defrost_conformal(engine, orc):
    """DEFROST split order (metric, drift, kick) with the spectral kick and expansion."""
    c = L.make_config(16, nfld=2, length=8.0, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                      split_order=L.SPLIT_DEFROST, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    g, o = pair(engine, orc, c)
    same_start(g, o, amp=0.05)
    for obj in (g, o):
        obj.set_scale_factor(1.0, 0.0)
        obj.calc_metric()
        obj.symp(6, 0.03, 4)
    compare_state(g, o)
    assert np.allclose(g.scale_factor(), o.scale_factor(), rtol=1e-11, atol=0)
    assert np.allclose(g.time(), o.time(), rtol=0, atol=1e-14)


def test_defrost_symp6_constant_and_symp8(engine, orc):
    """The DEFROST tree's own symp6 constant is used with its split order, and its
    symp8 (empty weights in the reference) is refused rather than run."""
    c = bubble_fd27(16, gw=False, split=L.SPLIT_DEFROST)
    g, o = pair(engine, orc, c)
    same_start(g, o, mean=0.0, amp=0.3)
    g.symp(6, 0.025, 3)
    o.symp(6, 0.025, 3)
    compare_state(g, o)
    assert np.allclose(g.time(), o.time(), rtol=0, atol=1e-15)
    with pytest.raises(engine.LatticeError):
        g.symp(8, 0.025, 1)


@pytest.mark.parametrize("shape,steps", [((64, 32, 32), 20), ((128, 128, 128), 4)])
def test_fp32_kahan_tracks_fp64_oracle(engine, orc, shape, steps):
    """The FP32-Kahan engine (cuFFT path and separable passes: the
    one-tile-per-block kind at 64x32x32, the streamed kind at 128^3) against
    the FP64 oracle."""
    nx, ny, nz = shape
    for impl in (L.SPEC_IMPL_CUFFT, L.SPEC_IMPL_SEPARABLE):
        c = L.make_config(shape, nfld=2, length=16.0 * nx / 64, laplacian=L.LAP_SPECTRAL,
                          background=L.BG_CONFORMAL, precision=L.FP32_KAHAN, model=L.MODEL_PHI4_G2,
                          model_params=(1.0, 2.0), spectral_impl=impl)
        g = engine.Lattice(c)
        if impl == L.SPEC_IMPL_SEPARABLE:
            assert g.sep_streamed() == (nx == 128)
        c64 = L.make_config(shape, nfld=2, length=16.0 * nx / 64, laplacian=L.LAP_SPECTRAL,
                            background=L.BG_CONFORMAL, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
        o = orc.Oracle(c64)
        f, p = random_state((2, nz, ny, nx), seed=17, mean=1.0, amp=0.01)
        for obj in (g, o):
            obj.set_state(f, p)
            obj.set_scale_factor(1.0, 0.0)
            obj.calc_metric()
            obj.symp(4, 0.02, steps)
        gf, gp = g.get_state()
        of, op = o.get_state()
        # fluctuations of ~1e-2 around 1: compare the fluctuation, not the mean;
        # FP32 rounding of fields near 1 is ~6e-8, i.e. ~1e-5 of the fluctuation
        assert rel_err(gf - 1.0, of - 1.0) <= 1e-4, impl
        assert rel_err(gp, op) <= 1e-4, impl
        assert abs(g.scale_factor()[0] - o.scale_factor()[0]) <= 1e-8 * o.scale_factor()[0]
