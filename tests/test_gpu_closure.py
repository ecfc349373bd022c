"""The learned closure on the GPU: BF16 tensor-core convolutions against the
CPU FP64 network oracle (forward and gradients), training, the sharp-k
coarsening against numpy FFTs, and the coupling of the network into the
coarse kick."""
from __future__ import annotations

import math

import numpy as np
import pytest

import net_oracle as NO
from conftest import rel_err
from helpers import L, random_state

pytestmark = pytest.mark.gpu


def _dataset(engine, shape, nsamp, seed):
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    host = rng.standard_normal((nsamp, 6, nz, ny, nx)).astype(np.float32)
    host[:, 0] += 0.5
    buf = engine.DeviceArray(host.size)
    buf.upload(host)
    return host, buf


def _net(engine, seed, scale_last=1.0):
    net = engine.Net(seed=seed)
    p = net.params()
    rng = np.random.default_rng(seed + 100)
    q = rng.standard_normal(p.size).astype(np.float32) * 0.2 * NO.mask().astype(np.float32)
    o = NO.unflatten(np.arange(p.size))
    q[o["W3"].astype(int).ravel()] *= scale_last
    net.set_params(q)
    norm = (np.array([0.5, 0.0, 0.0, 0.0]), np.array([1.0, 0.8, 1.2, 0.9]), np.array([1.5, 0.7]))
    net.set_norm(*norm)
    return net, q.astype(np.float64), norm


# (16, 8, 4): every layer on the mma.sync kernels; (128, 8, 2) and (64, 8, 5):
# the 4 -> 32 and 32 -> 32 layers (forward and backward data) on the tcgen05 /
# tensor-memory kernel, with 128-site x-rows and with two 64-site x-rows per
# M tile (five z-planes: one item's plane ring wraps)
SHAPES = [(16, 8, 4), (128, 8, 2), (64, 8, 5)]


@pytest.mark.parametrize("SHAPE", SHAPES)
def test_forward_matches_oracle(engine, SHAPE):
    host, buf = _dataset(engine, SHAPE, 3, 1)
    net, p, norm = _net(engine, 7)
    idx = [2, 0]
    out = net.forward(buf, 6 * int(np.prod(SHAPE)), idx, SHAPE)
    x = NO.pack_inputs(host[idx], norm[0], norm[1], emulate=True)
    ref_e, _ = NO.forward(p, x, emulate=True)
    ref, _ = NO.forward(p, NO.pack_inputs(host[idx], norm[0], norm[1]))
    scale = np.max(np.abs(ref))
    # FP32 accumulation against the emulated BF16 storage points: rounding flips only
    assert np.max(np.abs(out - ref_e)) <= 2e-2 * scale
    assert rel_err(out, ref_e) <= 5e-3
    # against the FP64 network: BF16 inputs, weights and activations
    assert rel_err(out, ref) <= 3e-2


@pytest.mark.parametrize("SHAPE", SHAPES)
def test_gradients_match_oracle(engine, SHAPE):
    """The hand-written backward kernels against the oracle's exact gradient."""
    host, buf = _dataset(engine, SHAPE, 2, 2)
    net, p, norm = _net(engine, 9)
    loss, g = net.grad(buf, 6 * int(np.prod(SHAPE)), [1, 0], SHAPE)
    lref_e, gref_e = NO.loss_and_grad(p, host[[1, 0]], norm, emulate=True)
    lref, gref = NO.loss_and_grad(p, host[[1, 0]], norm)
    assert abs(loss - lref_e) <= 1e-3 * lref_e
    assert abs(loss - lref) <= 2e-2 * lref
    off = 0
    for name, shp in NO.SHAPES:
        n = int(np.prod(shp))
        a, b, c = g[off:off + n], gref_e[off:off + n], gref[off:off + n]
        live = NO.mask()[off:off + n] > 0
        assert rel_err(a[live], b[live]) <= 2e-2, name
        assert rel_err(a[live], c[live]) <= 5e-2, name
        assert np.all(a[~live] == 0), name
        off += n


def test_training_reduces_loss(engine):
    """Adam steps of the GPU kernels fit a smooth target built from the inputs."""
    nx, ny, nz = 16, 16, 8
    rng = np.random.default_rng(5)
    k = 2 * np.pi * np.fft.fftfreq(nx)
    host = np.zeros((16, 6, nz, ny, nx), dtype=np.float32)
    for s in range(16):
        for c in range(4):  # smooth random fields
            f = rng.standard_normal((nz, ny, nx))
            F = np.fft.fftn(f)
            kk = np.sqrt(k[None, None, :] ** 2 + k[None, :, None] ** 2 + (2 * np.pi * np.fft.fftfreq(nz))[:, None, None] ** 2)
            F[kk > 1.2] = 0
            host[s, c] = np.real(np.fft.ifftn(F)) * 3
        phi, chi = host[s, 0], host[s, 1]
        host[s, 4] = phi * chi * chi
        host[s, 5] = phi * phi * chi
    buf = engine.DeviceArray(host.size)
    buf.upload(host)
    net = engine.Net(seed=3)
    net.set_norm([0, 0, 0, 0], [1 / host[:, c].std() for c in range(4)], [1 / host[:, 4].std(), 1 / host[:, 5].std()])
    stride = 6 * nx * ny * nz
    held = [14, 15]
    l0, _ = net.grad(buf, stride, held, (nx, ny, nz))
    for it in range(400):
        net.train_step(buf, stride, [it % 14, (it + 7) % 14], (nx, ny, nz), 3e-3 if it < 300 else 1e-3)
    l1, _ = net.grad(buf, stride, held, (nx, ny, nz))  # samples the network never saw
    assert l1 < 0.3 * l0, (l0, l1)


def test_coarsen_matches_numpy(engine):
    n, nc = 32, 16
    c = L.make_config(n, nfld=2, length=12.0, laplacian=L.LAP_SPECTRAL, precision=L.FP64,
                      model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    g = engine.Lattice(c)
    f, p = random_state((2, n, n, n), seed=8, mean=0.5, amp=0.3)
    g.set_state(f, p)
    buf = engine.DeviceArray(6 * nc ** 3)
    g.coarsen(nc, buf, 0, L.UNITS_PROGRAM)
    out = buf.download().reshape(6, nc, nc, nc).astype(np.float64)

    def filt(a):
        F = np.fft.rfftn(a) / a.size
        kz = np.fft.fftfreq(n, 1.0 / n)
        ky = kz
        kx = np.arange(n // 2 + 1)
        keep = (np.abs(kz)[:, None, None] < nc // 2) & (np.abs(ky)[None, :, None] < nc // 2) & (kx[None, None, :] < nc // 2)
        Fc = np.zeros((nc, nc, nc // 2 + 1), dtype=complex)
        sel = F * keep
        idx = np.r_[0:nc // 2, n - nc // 2 + 1:n]
        jdx = np.r_[0:nc // 2, nc // 2 + 1:nc]
        Fc[np.ix_(jdx, jdx, np.arange(nc // 2))] = sel[np.ix_(idx, idx, np.arange(nc // 2))]
        return np.fft.irfftn(Fc * nc ** 3, s=(nc, nc, nc))

    phic = [filt(f[i]) for i in range(2)]
    dv_f = [f[0] ** 3 + 2.0 * f[0] * f[1] ** 2, 2.0 * f[0] ** 2 * f[1]]
    dv_c = [phic[0] ** 3 + 2.0 * phic[0] * phic[1] ** 2, 2.0 * phic[0] ** 2 * phic[1]]
    refs = phic + [filt(p[i]) for i in range(2)] + [dv_c[i] - filt(dv_f[i]) for i in range(2)]
    for ch in range(6):
        # FP64 filter on the GPU, FP32 output
        assert np.max(np.abs(out[ch] - refs[ch])) <= 2e-6 * max(1.0, np.max(np.abs(refs[ch]))), ch
    g.close()


def test_zero_closure_matches_plain(engine):
    """A network that outputs zero leaves the evolution unchanged (to rounding)."""
    n = 32
    c = L.make_config((n, n, 16), nfld=2, length=16.0, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                      precision=L.FP64, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    f, p = random_state((2, 16, n, n), seed=4, mean=0.8, amp=0.1)
    net = engine.Net(seed=1)
    net.set_params(np.zeros(net.nparams, dtype=np.float32))
    res = []
    for attach in (False, True):
        g = engine.Lattice(c)
        g.set_state(f, p)
        g.set_scale_factor(1.0, 0.0)
        g.calc_metric()
        if attach:
            g.attach_closure(net, 1, L.UNITS_PROGRAM)
        g.symp(4, 0.02, 10)
        res.append((g.get_state(), g.scale_factor()))
        g.close()
    assert rel_err(res[0][0][0], res[1][0][0]) <= 1e-12
    assert rel_err(res[0][0][1], res[1][0][1]) <= 1e-11
    assert abs(res[0][1][0] - res[1][1][0]) <= 1e-12


def test_closure_force_enters_the_kick(engine):
    """A network with a constant output o adds hk a^4 o / out_scale to every
    momentum at every kick (Minkowski: a = 1): after a run the difference to
    the plain run is the summed kick sizes times the force, to first order."""
    n = 32
    c = L.make_config((n, 16, 16), nfld=2, length=16.0, laplacian=L.LAP_SPECTRAL, precision=L.FP64,
                      model=L.MODEL_FREE, model_params=(0.0,))
    f, p = random_state((2, 16, 16, n), seed=6, mean=0.0, amp=0.1)
    net = engine.Net(seed=1)
    q = np.zeros(net.nparams, dtype=np.float32)
    o = NO.unflatten(np.arange(net.nparams))
    q[int(o["b3"][0])] = 0.5
    q[int(o["b3"][1])] = -0.25
    net.set_params(q)
    net.set_norm([0, 0, 0, 0], [1, 1, 1, 1], [2.0, 4.0])
    res = []
    for attach in (False, True):
        g = engine.Lattice(c)
        g.set_state(f, p)
        if attach:
            g.attach_closure(net, 3, L.UNITS_PROGRAM)
        g.symp(2, 0.01, 10)  # leapfrog: 10 kicks of 0.01
        res.append(g.get_state())
        g.close()
    # massless free field: a uniform force only moves the k = 0 mode
    dpi = res[1][1] - res[0][1]
    assert np.allclose(dpi[0], 0.1 * 0.5 / 2.0, rtol=0, atol=1e-12)
    assert np.allclose(dpi[1], -0.1 * 0.25 / 4.0, rtol=0, atol=1e-12)


def test_closure_ablation_gain(engine):
    """What the trained network gains over the plain coarse method.

    Fine 64^3 runs with fluctuations up to the fine Nyquist wavenumber
    (<dphi^2> ~ 0.08) are filtered onto 16^3; three quarters of the variance
    lives in modes the coarse lattice cannot hold, and their mean-field force
    on the resolved modes is what the plain coarse kick misses.  After
    training on eight seeds, held-out seeds are evolved three ways from the
    same filtered state: the filtered fine run is the reference, and the
    closure must (a) explain most of the missing force on held-out samples
    and (b) bring the coarse P(k) (bins up to half the coarse Nyquist) closer
    to the reference than the plain coarse run."""
    import importlib
    C = importlib.import_module("lattice-dev_gb300.closure")
    s = C.Setup(n_fine=64, n_coarse=16, length=8.0, background=L.BG_MINKOWSKI, kcut_frac=1.0, amp=0.01,
                units=L.UNITS_PROGRAM)
    ds = C.generate(s, list(range(10, 18)), 0.5, 8.0, 20)
    net = engine.Net(seed=3)
    C.fit_norm(s, ds, net)
    order = np.random.default_rng(0).permutation(ds.count)
    hold, tr = order[:16], order[16:]
    C.train(s, ds, net, tr, epochs=40, batch=8, lr=3e-3, lr_end=3e-4)
    fe = C.force_error(s, ds, net, hold)  # the plain method has 1.0 by definition
    assert fe[0] < 0.2, fe
    assert fe[1] < 1.0, fe
    ev = C.evaluate(s, net, [70, 71, 72], 4.0, every=1)
    plain = np.mean([e["plain"]["pk_mean_rel_err"] for e in ev], axis=0)
    clos = np.mean([e["closure"]["pk_mean_rel_err"] for e in ev], axis=0)
    assert np.all(clos < 0.5 * plain), (plain, clos)
    ds.buf.close()


def test_attached_network_cannot_be_destroyed(engine):
    c = L.make_config((32, 16, 16), nfld=2, length=16.0, laplacian=L.LAP_SPECTRAL, model=L.MODEL_PHI4_G2,
                      model_params=(1.0, 2.0))
    g = engine.Lattice(c)
    net = engine.Net(seed=2)
    g.attach_closure(net, 1, L.UNITS_PROGRAM)
    with pytest.raises(engine.LatticeError) as ei:
        net.close()
    assert ei.value.code == 6  # LAT_ERR_STATE
    g.attach_closure(None)
    net.close()  # detached: freed
    g.close()


def test_closure_graphs_keyed_on_network_state(engine):
    """Graphs of lat_symp are cached per closure state: a graph prepared with
    the network attached is replayed after a detach and re-attach, and a new
    normalisation (captured by value in the graph) is never replayed stale."""
    c = L.make_config((32, 16, 16), nfld=2, length=16.0, laplacian=L.LAP_SPECTRAL, precision=L.FP64,
                      model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    f, p = random_state((2, 16, 16, 32), seed=13, mean=0.5, amp=0.2)
    net = engine.Net(seed=5)
    q = np.random.default_rng(1).standard_normal(net.nparams).astype(np.float32) * 0.05
    net.set_params(q)
    norm_a = ([0.5, 0.0, 0.0, 0.0], [1.0, 1.0, 1.0, 1.0], [2.0, 3.0])
    norm_b = ([0.5, 0.0, 0.0, 0.0], [1.0, 1.0, 1.0, 1.0], [0.5, 0.25])

    def run(prepare, norm):
        g = engine.Lattice(c)
        g.set_state(f, p)
        net.set_norm(*norm_a)
        if prepare:  # graph built with the closure attached, then detached
            g.attach_closure(net, 2, L.UNITS_PROGRAM)
            g.prepare_symp(2, 0.02, 6)
            g.attach_closure(None)
        net.set_norm(*norm)
        g.attach_closure(net, 2, L.UNITS_PROGRAM)
        l0 = g.launch_count()
        g.symp(2, 0.02, 6)
        out = g.get_state(), g.launch_count() - l0
        g.attach_closure(None)
        g.close()
        return out

    fresh_a, _ = run(False, norm_a)
    fresh_b, _ = run(False, norm_b)
    assert not np.array_equal(fresh_a[1], fresh_b[1])  # the normalisation matters
    replay_a, _ = run(True, norm_a)
    assert np.array_equal(replay_a[0], fresh_a[0]) and np.array_equal(replay_a[1], fresh_a[1])
    renorm, _ = run(True, norm_b)  # prepared under norm_a: must not be replayed
    assert np.array_equal(renorm[0], fresh_b[0]) and np.array_equal(renorm[1], fresh_b[1])
    net.close()


def test_closure_side_stream_matches_in_order(engine):
    """The network runs on a side stream beside the kick's transforms and is
    joined before the fused kick+drift; timed (eager, in-order) launches
    must give the same bits.  Conformal background, conformal units (the
    network sees a after the group's first gravity half-step)."""
    c = L.make_config((32, 16, 16), nfld=2, length=16.0, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                      precision=L.FP32_KAHAN, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))
    f, p = random_state((2, 16, 16, 32), seed=21, mean=0.6, amp=0.2)
    net = engine.Net(seed=8)
    net.set_params(np.random.default_rng(3).standard_normal(net.nparams).astype(np.float32) * 0.05)
    net.set_norm([0.5, 0.0, 0.0, 0.0], [1.0, 1.0, 1.0, 1.0], [1.5, 2.5])
    out = []
    for timed in (False, True):
        g = engine.Lattice(c)
        g.set_state(f, p)
        g.set_scale_factor(1.0, 0.0)
        g.calc_metric()
        g.attach_closure(net, 2, L.UNITS_CONFORMAL)
        g.timing(timed)
        g.symp(4, 0.02, 5)
        out.append((g.get_state(), g.scale_factor()))
        g.attach_closure(None)
        g.close()
    (fa, pa), sa = out[0]
    (fb, pb), sb = out[1]
    assert np.array_equal(fa, fb) and np.array_equal(pa, pb) and sa == sb
    net.close()
