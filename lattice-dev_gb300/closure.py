"""Learned subgrid closure for coarse two-field preheating lattices.

Pipeline (all compute on the GPU through the C ABI; numpy only moves small
host arrays):

1. ``generate``: fine-lattice runs of the two-field model
   V = phi^4/4 + g2 phi^2 chi^2/2 from seeded vacuum fluctuations; at each
   snapshot ``lat_coarsen`` writes the sharp-k filtered coarse fields,
   momenta and the force the coarse kick misses,
   Delta_f = V'_f(F phi) - F V'_f(phi), into one device data set.
2. ``fit_norm`` / ``train``: the network (lat_net_*) is trained by its own
   BF16 forward and backward kernels with Adam to predict Delta from
   (phi, chi, pi_phi, pi_chi) on the coarse lattice.
3. ``evaluate``: held-out seeds evolved three ways from the same initial
   state: the fine lattice (filtered for comparison), the plain coarse
   lattice, and the coarse lattice with the closure attached; the power
   spectra of phi and chi up to half the coarse Nyquist wavenumber are
   compared with the filtered fine run.

The closure has no counterpart in the reference; the fine and coarse
evolutions are the reference's spectral Yoshida-4 step
(Pseudospec/openmp_dev/evolve_spectral.f90:129-227).
"""
from __future__ import annotations

import importlib
import math
import time
from dataclasses import dataclass, field

import numpy as np

L = importlib.import_module("lattice-dev_gb300")

CHANNELS = 6  # phi, chi, pi_phi, pi_chi, Delta_phi, Delta_chi


@dataclass
class Setup:
    n_fine: int = 256
    n_coarse: int = 64
    length: float = 10 * math.pi
    g2: float = 2.0
    amp: float = 1e-8
    dt_frac: float = 20.0  # dt = dx / dt_frac on each lattice
    order: int = 4
    fine_precision: int = L.FP32_KAHAN
    background: int = L.BG_CONFORMAL
    kcut_frac: float = 0.5  # initial fluctuations up to this fraction of the fine Nyquist wavenumber
    units: int = L.UNITS_CONFORMAL  # variables of the training data and of the attached closure
    tune_cache: str | None = None  # autotuner cache shared by the fine runs (None: tune every handle)

    def config(self, n, precision, impl=L.SPEC_IMPL_AUTO):
        return L.make_config(n, nfld=2, length=self.length, laplacian=L.LAP_SPECTRAL, background=self.background,
                             precision=precision, model=L.MODEL_PHI4_G2, model_params=(1.0, self.g2),
                             spectral_impl=impl)

    def dt(self, n):
        return self.length / n / self.dt_frac

    @property
    def nsite(self):
        return self.n_coarse ** 3

    @property
    def stride(self):
        return CHANNELS * self.nsite


def init_fine(s: Setup, g, seed):
    g.init_vacuum(seed, [1.0, 0.0], [0.0, 0.0], [3.0, s.g2], amp=s.amp, kcut_frac=s.kcut_frac)
    if s.background == L.BG_CONFORMAL:
        g.set_scale_factor(1.0, 0.0)
        g.calc_metric()


def coarse_state(s: Setup, fine, scratch: L.DeviceArray):
    """Filtered (fields, momenta, Delta) of a fine lattice as FP64 host arrays on the
    coarse grid, in the evolved (program) variables."""
    fine.coarsen(s.n_coarse, scratch, 0, L.UNITS_PROGRAM)
    n = s.n_coarse
    a = scratch.download(CHANNELS * s.nsite).astype(np.float64).reshape(CHANNELS, n, n, n)
    return a[0:2].copy(), a[2:4].copy(), a[4:6].copy()


@dataclass
class DataSet:
    buf: L.DeviceArray
    count: int
    meta: list = field(default_factory=list)  # (seed, time) per sample


def generate(s: Setup, seeds, t_start, t_end, n_snap, capacity=None, progress=None) -> DataSet:
    """Snapshots of fine runs, n_snap per seed evenly in [t_start, t_end]."""
    cap = capacity or len(seeds) * n_snap
    buf = L.DeviceArray(cap * s.stride)
    ds = DataSet(buf, 0)
    dt = s.dt(s.n_fine)
    times = np.linspace(t_start, t_end, n_snap)
    for seed in seeds:
        g = L.Lattice(s.config(s.n_fine, s.fine_precision))
        init_fine(s, g, seed)
        g.autotune(s.tune_cache)
        done = 0
        for t in times:
            k = int(round(t / dt)) - done
            if k > 0:
                g.symp(s.order, dt, k)
                done += k
            g.coarsen(s.n_coarse, buf, ds.count * s.stride, s.units)
            ds.meta.append((seed, done * dt))
            ds.count += 1
        g.close()
        if progress:
            progress(seed)
    return ds


def fit_norm(s: Setup, ds: DataSet, net, nsamp=8):
    """Input shift/scale and output scale from a subset of the samples."""
    idx = np.linspace(0, ds.count - 1, min(nsamp, ds.count)).astype(int)
    acc = [[] for _ in range(CHANNELS)]
    for i in idx:
        a = ds.buf.download(s.stride, i * s.stride).reshape(CHANNELS, -1)
        for c in range(CHANNELS):
            acc[c].append(a[c].astype(np.float64))
    arr = [np.concatenate(v) for v in acc]
    shift = np.array([0.0, 0.0, 0.0, 0.0])  # phi oscillates about zero; keep the sign information
    scale = np.array([1.0 / max(np.sqrt(np.mean(arr[c] ** 2)), 1e-30) for c in range(4)])
    oscale = np.array([1.0 / max(np.std(arr[4 + c]), 1e-30) for c in range(2)])
    net.set_norm(shift, scale, oscale)
    return shift, scale, oscale


def train(s: Setup, ds: DataSet, net, train_idx, epochs=20, batch=4, lr=2e-3, lr_end=2e-4, seed=0, log=None):
    rng = np.random.default_rng(seed)
    shape = (s.n_coarse, s.n_coarse, s.n_coarse)
    tr = np.asarray(train_idx)
    nb = max(1, len(tr) // batch)
    total = epochs * nb
    hist = []
    step = 0
    for ep in range(epochs):
        perm = rng.permutation(tr)
        losses = []
        for b in range(nb):
            frac = step / max(total - 1, 1)
            rate = lr * (lr_end / lr) ** frac  # geometric decay
            losses.append(net.train_step(ds.buf, s.stride, perm[b * batch:(b + 1) * batch], shape, rate))
            step += 1
        hist.append(float(np.mean(losses)))
        if log:
            log(ep, hist[-1])
    return hist


def force_error(s: Setup, ds: DataSet, net, idx):
    """Held-out relative force error: |Delta - Delta_net|^2 / |Delta|^2 per channel
    (1.0 is the plain coarse method, which uses Delta = 0)."""
    shape = (s.n_coarse,) * 3
    _, _, oscale = net.norm()
    num = np.zeros(2)
    den = np.zeros(2)
    for i in idx:
        out = net.forward(ds.buf, s.stride, [i], shape)[0]
        a = ds.buf.download(s.stride, i * s.stride).reshape(CHANNELS, *shape)
        for c in range(2):
            pred = out[..., c] / oscale[c]
            num[c] += np.sum((a[4 + c].astype(np.float64) - pred) ** 2)
            den[c] += np.sum(a[4 + c].astype(np.float64) ** 2)
    return num / den


def spectra(s: Setup, fields, momenta, nbins):
    """P(k) of phi and chi on the coarse grid (weighted binning), through an FP64 coarse handle."""
    h = L.Lattice(s.config(s.n_coarse, L.FP64))
    h.set_state(fields, momenta)
    out = [h.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, nbins)[0] for f in (0, 1)]
    h.close()
    return np.array(out)


def pk_error(S, Sref, kmax_bin):
    rel = np.abs(S[:, 1:kmax_bin] - Sref[:, 1:kmax_bin]) / np.maximum(np.abs(Sref[:, 1:kmax_bin]), 1e-300)
    return rel.max(axis=1), rel.mean(axis=1)


def evaluate(s: Setup, net, seeds, t_eval, every=3, coarse_precision=L.FP32_KAHAN, nbins=None, t_attach=0.0):
    """Fine, plain coarse and closure coarse runs of held-out seeds; P(k) errors
    up to half the coarse Nyquist wavenumber and times to solution.  The
    closure is attached from t_attach on (the start of its training window)."""
    n = s.n_coarse
    nbins = nbins or n // 2
    # bins of width dk (the fundamental): half the coarse Nyquist is n/4 bins
    kmax_bin = n // 4
    scratch = L.DeviceArray(s.stride)
    res = []
    for seed in seeds:
        f = L.Lattice(s.config(s.n_fine, s.fine_precision))
        init_fine(s, f, seed)
        f.autotune(s.tune_cache)  # the fine reference runs on the engine's fastest path for its lattice
        fld0, mom0, _ = coarse_state(s, f, scratch)
        dtf = s.dt(s.n_fine)
        kf = int(round(t_eval / dtf))
        f.prepare_symp(s.order, dtf, kf)  # graph built outside the timed region
        f.sync()
        f.mark(0)
        f.symp(s.order, dtf, kf)
        f.mark(1)
        t_fine = f.mark_elapsed(0, 1) * 1e-3
        fldT, momT, _ = coarse_state(s, f, scratch)
        S_ref = spectra(s, fldT, momT, nbins)
        f.close()
        dtc = s.dt(n)
        kc = int(round(t_eval / dtc))
        runs = {}
        k1 = min(kc, int(round(t_attach / dtc)))
        for name, attach in (("plain", False), ("closure", True)):
            c = L.Lattice(s.config(n, coarse_precision, L.SPEC_IMPL_CUFFT))
            c.set_state(fld0, mom0)
            if s.background == L.BG_CONFORMAL:
                c.set_scale_factor(1.0, 0.0)
                c.calc_metric()
            # both segments' graphs built outside the timed region (the
            # second with the network attached: the graph cache keys on it)
            if k1:
                c.prepare_symp(s.order, dtc, k1)
            if kc - k1:
                if attach:
                    c.attach_closure(net, every, s.units)
                c.prepare_symp(s.order, dtc, kc - k1)
                if attach:
                    c.attach_closure(None)
            c.sync()
            c.mark(0)
            if k1:
                c.symp(s.order, dtc, k1)
            if attach:
                c.attach_closure(net, every, s.units)
            if kc - k1:
                c.symp(s.order, dtc, kc - k1)
            c.mark(1)
            tc = c.mark_elapsed(0, 1) * 1e-3
            fl, mo = c.get_state()
            S = spectra(s, fl, mo, nbins)
            mx, mean = pk_error(S, S_ref, kmax_bin)
            runs[name] = {"time_s": tc, "pk_max_rel_err": mx.tolist(), "pk_mean_rel_err": mean.tolist()}
            c.close()
        res.append({"seed": seed, "t": kf * dtf, "fine_time_s": t_fine, **runs})
    scratch.close()
    return res
