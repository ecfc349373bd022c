#!/usr/bin/env python
"""Benchmark of the GB300 lattice engine.

Workload (the headline configuration): two-field preheating
V = phi^4/4 + g2 phi^2 chi^2/2 (g2 = 2) on a 256^3 lattice, L = 10 pi,
pseudospectral Laplacian, self-consistent conformal expansion from a(0) = 1,
4th-order Yoshida with dt = dx/20, FP32 fields with Kahan-compensated drifts
and FP64 reductions.  A step is one Yoshida-4 step (three kicks and three
drifts) of the whole lattice; the metric is site-updates/s (lattice sites x
steps / s).  Inputs are vacuum fluctuations drawn on the device (seeded).

Reported beside it: the FP64 plain step on the GPU, the accuracy of the
FP32-Kahan run against that FP64 run, the roofline of the dominant engine
kernel (CUDA events on the engine's stream), an end-to-end number through the
C ABI with host arrays, and the CPU restatement of the reference on the host
cores.

``--impl reference`` times the CPU restatement of the reference algorithm
(the reference is Fortran + FFTW and cannot be built here) on all host cores.
"""
from __future__ import annotations

import argparse
import importlib
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for p in (str(ROOT), str(ROOT / "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "site-updates/s @256^3 two-field spectral Yoshida-4, FP32-Kahan"
UNIT = "site-updates/s"
N_SIDE = 256
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}


def workload_config(L, precision, n=N_SIDE, impl=0):
    return L.make_config(n, nfld=2, length=10 * math.pi, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                         precision=precision, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0), spectral_impl=impl)


def init_state(obj, seed):
    obj.init_vacuum(seed, [1.0, 0.0], [0.0, 0.0], [3.0, 2.0], amp=1e-8, kcut_frac=0.5)
    obj.set_scale_factor(1.0, 0.0)  # a(0) = 1, then ysclp from the Friedmann constraint
    obj.calc_metric()


def ncu_traffic(kernel_class, workload="spectral256_2f_fp32"):
    """DRAM bytes (read + write) per launch of a kernel class from the committed ncu capture, or None."""
    p = ROOT / "profiles" / "dram_traffic_256cube.txt"
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        f = ln.split()
        if len(f) >= 4 and not ln.startswith("#") and f[0] == kernel_class and f[1] == workload:
            return float(f[2]) + float(f[3])
    return None


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def stop(self, t0=None, t1=None):
        """Summary of the samples that arrived in [t0, t1] (host monotonic
        clock, 50 ms on both sides: a few sample intervals), or of all samples."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        lines = [ln for t, ln in self.lines if t0 is None or (t0 - 0.05 <= t <= t1 + 0.05)]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ cpu leg
def cpu_rate(steps_budget_s=20.0, max_steps=None, n=N_SIDE, warmup=1):
    """Times the CPU restatement (FP64, OpenMP on all host cores) on Yoshida-4
    steps of the same workload after `warmup` untimed steps; returns
    (site-updates/s, cores, steps, seconds)."""
    import py_oracle
    L = importlib.import_module("lattice-dev_gb300")
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    c = workload_config(L, L.FP64, n)
    o = py_oracle.Oracle(c)
    init_state(o, 1000)
    dt = c.len / n / 20
    o.symp(4, dt, max(warmup, 1))  # warm-up (first-touch, FFT twiddles)
    done, t0 = 0, time.perf_counter()
    while True:
        o.symp(4, dt, 1)
        done += 1
        el = time.perf_counter() - t0
        if el >= steps_budget_s or (max_steps and done >= max_steps):
            break
    return n ** 3 * done / el, int(os.environ.get("OMP_NUM_THREADS", cores)), done, el


def run_reference(args):
    ws, rank, _, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0, None
    if rank != 0:
        return 0
    try:
        import py_oracle
        py_oracle.load()
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": f"CPU restatement could not be built: {e}"}))
        return 0
    budget = float(os.environ.get("LAT_REF_BUDGET_S", "60"))
    warm = max(args.warmup, 1)
    rate, cores, done, el = cpu_rate(steps_budget_s=budget, max_steps=max(args.steps, 1), warmup=warm)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT,
        "n_gpus": ws, "steps": done, "warmup": warm, "ms_per_step": 1e3 * el / done, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded vacuum fluctuations)",
        "config": {"workload": "two-field preheating 256^3, L=10pi, spectral, Yoshida-4, conformal, dt=dx/20",
                   "global_batch": N_SIDE ** 3, "seq_len": 1, "parallelism": "replicas"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{done} Yoshida-4 steps of the 256^3 workload after {warm} warm-up steps "
                                   "(CPU restatement of the Fortran reference, FP64, OpenMP; the reference "
                                   "itself needs a Fortran compiler and FFTW, absent here)"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ gpu leg
def run_ours(args):
    ws, rank, local, pg = dist_setup()
    L = importlib.import_module("lattice-dev_gb300")
    L.load_library()
    K, W = args.steps, args.warmup
    sampler = ClockSampler(local)  # sampling long before the timed region, which keeps its own window
    if args.case == "headline":
        sampler.start()
    if args.case == "fd-bubbles":
        return run_fd_case(L, args, local)
    if args.case == "closure":
        return run_closure_case(L, args, local)
    if args.case == "ensemble":
        return run_ensemble_case(L, args)
    if args.case == "conv":
        return run_conv_case(L, args, local)
    n = args.n or N_SIDE
    impl = {"auto": L.SPEC_IMPL_AUTO, "cufft": L.SPEC_IMPL_CUFFT, "separable": L.SPEC_IMPL_SEPARABLE}[args.spectral_impl]
    c = workload_config(L, L.FP32_KAHAN, n, impl)
    c.device = local
    g = L.Lattice(c)
    N = n ** 3
    dt = c.len / n / 20
    init_state(g, 1000 + rank)
    # tile shapes, launch shapes and (with spectral_impl auto) the spectral path
    # picked by the autotuner on this lattice; the state is restored afterwards
    if not args.no_autotune:
        g.autotune(os.environ.get("LAT_TUNE_CACHE"))
    tuning = g.tuning()

    # warm-up, and the CUDA graph of the timed call built outside the timed region
    g.symp(4, dt, W)
    g.prepare_symp(4, dt, K)
    g.sync()

    # timed region: exactly K Yoshida-4 steps in one symp4(dt, K) call; the
    # clock sampler (started with the run) keeps the samples of this window
    barrier(pg)
    g.sync()
    l0 = g.launch_count()
    tr0 = time.monotonic()
    g.mark(0)
    g.symp(4, dt, K)
    g.mark(1)
    g.sync()
    tr1 = time.monotonic()
    barrier(pg)
    ms = g.mark_elapsed(0, 1)
    launches = g.launch_count() - l0
    clocks = sampler.stop(tr0, tr1)
    ms = max_over_ranks(pg, ms)
    value = ws * N * K / (ms * 1e-3)

    extra = {}
    if rank == 0 and not args.quick and n == N_SIDE:
        args.device_index = local
        extra = diagnostics(L, g, args, dt, ms / K)
    g.close()

    if rank != 0:
        return 0
    pk, pk_kind = peaks()
    line = {
        "metric": METRIC if n == N_SIDE else METRIC.replace("256^3", f"{n}^3"),
        "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (Kahan-compensated drifts, f64 reductions)",
        "data": "synthetic (seeded vacuum fluctuations, 1e-8/(2w_k) spectrum)",
        "config": {"workload": f"two-field preheating {n}^3, L=10pi, spectral, Yoshida-4, conformal, dt=dx/20",
                   "global_batch": N * ws, "seq_len": 1, "parallelism": f"replicas x{ws}",
                   "l2": "inputs larger than L2 (state 403 MB + spectra 270 MB per replica)"
                         if n == N_SIDE else "small profiling case",
                   "tuning": list(tuning),
                   "spectral_path": "separable passes" if tuning[5] == L.SPEC_IMPL_SEPARABLE else "cuFFT 3D"},
        "clocks": clocks, "gpu_launches": launches,
    }
    line.update(extra)
    if "roofline" in line and line["roofline"]:
        line["roofline"]["peak_kind"] = pk_kind
    print(json.dumps(line))
    return 0


def diagnostics(L, g, args, dt, ms_step):
    out = {}
    pk, pk_kind = peaks()
    hbm = float(pk.get("hbm_gbs", 6800.0))
    n = N_SIDE
    N = n ** 3
    # ---- per-kernel-class timing (eager launches, events per launch)
    Kt = max(4, min(args.steps, 20))
    g.timing(True)
    g.timing_reset()
    g.symp(4, dt, Kt)
    g.sync()
    cls = {}
    names = {L.K_KICKDRIFT: "kickdrift", L.K_DRIFT: "drift", L.K_KICK: "kick", L.K_KMUL: "kmul",
             L.K_FFT_R2C: "cufft_r2c", L.K_FFT_C2R: "cufft_c2r", L.K_OTHER: "other",
             L.K_SEP_X: "sep_x", L.K_SEP_Y: "sep_y", L.K_SEP_Z: "sep_z"}
    for k, nm in names.items():
        t, nl = g.timing_read(k)
        if nl:
            cls[nm] = {"ms": t, "launches": nl, "avg_us": 1e3 * t / nl}
    g.timing(False)
    tot = sum(v["ms"] for v in cls.values()) or 1.0
    for v in cls.values():
        v["share"] = v["ms"] / tot
    out["kernel_classes"] = cls
    # algorithmic bytes per launch of the engine kernels, two FP32 fields.
    # Streamed separable passes: X r phi,c,pi w phi,c,zs,pi; Y r zs,pi w pi; Z r zs,pi w pi.
    # Other separable passes: X r phi,c,pi w phi,c,lap; Y r phi,c,lap w lap; Z r phi,c,lap,pi w pi.
    streamed = g.sep_streamed()
    sep_b = (28, 12, 12) if streamed else (24, 16, 20)
    bytes_per = {"kickdrift": 2 * 28 * N, "kmul": 2 * 2 * 8 * (n // 2 + 1) * n * n, "drift": 2 * 20 * N,
                 "sep_x": 2 * sep_b[0] * N, "sep_y": 2 * sep_b[1] * N, "sep_z": 2 * sep_b[2] * N}
    own = {k: v for k, v in cls.items() if k in bytes_per}
    if own:
        dom = max(own, key=lambda k: own[k]["ms"])
        avg_s = own[dom]["avg_us"] * 1e-6
        ach = bytes_per[dom] / avg_s / 1e9
        out["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm, "unit": "GB/s",
                           "frac": ach / hbm,
                           "traffic": ncu_traffic(dom, "spectral256_2f_fp32_streamed" if streamed and
                                                  dom.startswith("sep") else "spectral256_2f_fp32"),
                           "algorithmic_bytes_per_launch": bytes_per[dom],
                           "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, "
                                             "same workload (profiles/dram_traffic_256cube.txt)"}
    # ---- both spectral paths: step time and FP32 accuracy
    paths = {}
    for impl, name in ((L.SPEC_IMPL_CUFFT, "cufft"), (L.SPEC_IMPL_SEPARABLE, "separable")):
        gp = L.Lattice(workload_config(L, L.FP32_KAHAN, impl=impl))
        init_state(gp, 1000)
        gp.symp(4, dt, 3)
        Kp = max(10, args.steps // 4)
        gp.sync()
        gp.mark(0)
        gp.symp(4, dt, Kp)
        gp.mark(1)
        msp = gp.mark_elapsed(0, 1) / Kp
        paths[name] = {"ms_per_step": msp, "value": N / (msp * 1e-3)}
        gp.close()
    out["spectral_paths"] = paths
    # each path's whole step against its own byte model: the cuFFT path moves
    # 3 kicks x (2 fields x (r2c + c2r: N reals + M complex each) + 28 B/site/field);
    # the streamed separable passes 3 kicks x 2 fields x (28 + 12 + 12) B/site
    # (the others 24 + 16 + 20)
    M = (n // 2 + 1) * n * n
    fft_bytes = 3 * (2 * (2 * 4 * N + 2 * 8 * M) + 2 * 28 * N)
    sep_bytes = 3 * 2 * (52 if streamed else 60) * N
    out["step_roofline"] = {
        "cufft": {"bytes_per_step": fft_bytes, "ms_per_step": paths["cufft"]["ms_per_step"],
                  "achieved_gbs": fft_bytes / (paths["cufft"]["ms_per_step"] * 1e-3) / 1e9},
        "separable": {"bytes_per_step": sep_bytes, "ms_per_step": paths["separable"]["ms_per_step"],
                      "achieved_gbs": sep_bytes / (paths["separable"]["ms_per_step"] * 1e-3) / 1e9},
        "note": "a 3D transform is counted as one read and one write of its input and output"}
    # the headline step against the byte model of a fused spectral kick+drift
    # path: per kick and field one R2C and one C2R (each one read of its input
    # and one write of its output: 2 (4N + 8M) B) plus 28 B/site of pass
    # arrays (phi, c, pi, lap read; phi, c, pi written): 264.4 B/site-update
    # at 256^3, whichever path runs
    out["step_roofline"]["survey_model"] = {
        "bytes_per_step": fft_bytes, "bytes_per_site_update": fft_bytes / N, "ms_per_step": ms_step,
        "achieved_gbs": fft_bytes / (ms_step * 1e-3) / 1e9,
        "note": "headline ms_per_step against 3 kicks x 2 fields x (2 (4N + 8M) + 28N) bytes"}
    for v in out["step_roofline"].values():
        if isinstance(v, dict):
            v["frac"] = v["achieved_gbs"] / hbm
    # ---- a longer timed region on the headline handle (clock samples over ~1 s)
    Ks = args.sustained_steps
    if Ks > 0:
        smp = ClockSampler(args.device_index)
        smp.start()  # nvidia-smi starts while the graph is built
        g.prepare_symp(4, dt, Ks)
        g.symp(4, dt, 3)
        g.sync()
        t0 = time.monotonic()
        g.mark(0)
        g.symp(4, dt, Ks)
        g.mark(1)
        g.sync()
        t1 = time.monotonic()
        msK = g.mark_elapsed(0, 1)
        out["sustained"] = {"steps": Ks, "ms_per_step": msK / Ks, "value": N * Ks / (msK * 1e-3),
                            "clocks": smp.stop(t0, t1)}
    # ---- FP64 plain step on the GPU
    if not args.no_fp64:
        c64 = workload_config(L, L.FP64)
        g64 = L.Lattice(c64)
        init_state(g64, 1000)
        g64.symp(4, dt, 2)
        K64 = max(3, args.steps // 4)
        g64.sync()
        g64.mark(0)
        g64.symp(4, dt, K64)
        g64.mark(1)
        ms64 = g64.mark_elapsed(0, 1) / K64
        out["fp64_plain"] = {"ms_per_step": ms64, "value": N / (ms64 * 1e-3), "steps": K64,
                             "fp32_kahan_speedup": ms64 / ms_step}
        # ---- accuracy of FP32-Kahan (both spectral paths) against the FP64 GPU run from the same IC
        steps_acc = args.acc_steps
        b64 = g64
        init_state(b64, 4242)
        e0 = b64.energies()
        b64.symp(4, dt, steps_acc)
        e64 = b64.energies()
        nb = 128
        S64 = [b64.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, nb)[0] for f in (0, 1)]
        accs = {}
        for impl, name in ((L.SPEC_IMPL_CUFFT, "cufft"), (L.SPEC_IMPL_SEPARABLE, "separable")):
            a32 = L.Lattice(workload_config(L, L.FP32_KAHAN, impl=impl))
            init_state(a32, 4242)
            a32.symp(4, dt, steps_acc)
            e32 = a32.energies()
            acc = {"steps": steps_acc}
            for f in (0, 1):
                S32, _ = a32.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, nb)
                live = np.arange(nb) >= 1
                rel = np.abs(S32[live] - S64[f][live]) / np.maximum(np.abs(S64[f][live]), 1e-300)
                acc[f"pk_field{f}_max_rel_err"] = float(np.max(rel[: n // 4]))
            acc["a_rel_err"] = abs(e32[L.E_A] - e64[L.E_A]) / e64[L.E_A]
            acc["energy_rel_err"] = abs(e32[L.E_RHO] - e64[L.E_RHO]) / abs(e64[L.E_RHO])
            acc["friedmann_residual_fp32"] = float(e32[L.E_RESIDUAL])
            accs[name] = acc
            a32.close()
        accs["friedmann_residual_fp64"] = float(e64[L.E_RESIDUAL])
        accs["friedmann_residual_initial"] = float(e0[L.E_RESIDUAL])
        out["accuracy_vs_fp64_gpu"] = accs
        g64.close()
    # ---- end to end through the C ABI with pinned host arrays (Fortran layout)
    sub = args.e2e_sub
    nf = 2
    nbytes = nf * N * 8
    hf = L.host_alloc(nbytes)
    hp = L.host_alloc(nbytes)
    import ctypes
    fa = np.ctypeslib.as_array((ctypes.c_double * (nf * N)).from_address(hf)).reshape(n, n, n, nf)
    pa = np.ctypeslib.as_array((ctypes.c_double * (nf * N)).from_address(hp)).reshape(n, n, n, nf)
    g.download_fortran(fa, 0, 0, pa, 0, 0)
    reps = max(2, args.e2e_reps)
    g.upload_fortran(fa, 0, 0, pa, 0, 0)
    g.symp(4, dt, sub)
    g.energies()
    g.download_fortran(fa, 0, 0, pa, 0, 0)
    t0 = time.perf_counter()
    for _ in range(reps):
        g.upload_fortran(fa, 0, 0, pa, 0, 0)
        g.symp(4, dt, sub)
        g.energies()
        g.download_fortran(fa, 0, 0, pa, 0, 0)
    el = time.perf_counter() - t0
    tu = td = te = 0.0
    for _ in range(reps):
        t1 = time.perf_counter()
        g.upload_fortran(fa, 0, 0, pa, 0, 0)
        t2 = time.perf_counter()
        g.symp(4, dt, sub)
        g.energies()
        t3 = time.perf_counter()
        g.download_fortran(fa, 0, 0, pa, 0, 0)
        t4 = time.perf_counter()
        tu, te, td = tu + t2 - t1, te + t3 - t2, td + t4 - t3
    L.host_free(hf)
    L.host_free(hp)
    out["e2e"] = {"value": N * sub * reps / el, "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes / sub,
                  "d2h_bytes_per_step": (2 * nbytes + 8 * L.NENERGY) / sub,
                  "steps_per_call": sub, "calls": reps,
                  "ms_per_call": {"upload": 1e3 * tu / reps, "symp_and_energies": 1e3 * te / reps,
                                  "download": 1e3 * td / reps},
                  "host_copy_share": (tu + td) / (tu + td + te),
                  "call": f"lat_upload + lat_symp(4, dt, {sub}) + lat_energies + lat_download "
                          "(FP64 Fortran-layout pinned host arrays, host clock around the calls)"}
    # ---- the other workloads of the engine (FD stencil paths, batched ensemble)
    if not args.no_fd:
        out["fd_workloads"] = fd_workloads(L, hbm)
        out["ensemble"] = ensemble_workload(L, 100)
    # ---- the learned closure on the preheating model (a reduced form of the closure benchmark)
    if not args.no_closure:
        out["closure"] = closure_workload(L, args)
    # ---- CPU restatement on the host cores
    if not args.no_cpu:
        rate, cores, done, el = cpu_rate(steps_budget_s=args.cpu_budget, max_steps=args.cpu_steps)
        out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": f"{done} Yoshida-4 steps of the same 256^3 workload in FP64 "
                                         f"({el:.1f} s) after 1 warm-up step; CPU restatement of the "
                                         "Fortran reference, OpenMP"}
    return out


def closure_workload(L, args):
    """The learned closure on the two-field preheating model of the headline
    (V = phi^4/4 + g2 phi^2 chi^2/2, g2 = 2, L = 10 pi, conformal, Yoshida-4,
    dt = dx/20 on each lattice), fine lattice filtered 4x (sharp k) to the
    coarse one, evolved to the headline workload's horizon (5000 steps of the
    256^3 lattice, t = 30.7).  Training data from --closure-train-seeds fine
    runs (snapshots from t = 5), the network trained by its own BF16 kernels,
    then --closure-eval-seeds held-out seeds evolved fine, plain coarse and
    coarse with the closure: P(k) errors of phi and chi against the filtered
    fine run up to half the coarse Nyquist wavenumber, and times to solution
    (CUDA events around each evolution).  The full benchmark's sizes (512^3 ->
    128^3, 64 + 16 seeds) are `--case closure` arguments."""
    import tempfile
    C = importlib.import_module("lattice-dev_gb300.closure")
    nf, nc = args.closure_n_fine, args.closure_n_fine // 4
    tune = tempfile.NamedTemporaryFile(prefix="lat_tune_", suffix=".jsonl", delete=False).name
    s = C.Setup(n_fine=nf, n_coarse=nc, tune_cache=tune)
    t_end = 5000 * s.dt(256)
    train_seeds = list(range(100, 100 + args.closure_train_seeds))
    eval_seeds = list(range(900, 900 + args.closure_eval_seeds))
    t0 = time.perf_counter()
    ds = C.generate(s, train_seeds, 5.0, t_end, 9)
    t_gen = time.perf_counter() - t0
    net = L.Net(seed=11)
    C.fit_norm(s, ds, net)
    order = np.random.default_rng(0).permutation(ds.count)
    n_hold = max(1, ds.count // 8)
    hold, tr = order[:n_hold], order[n_hold:]
    t0 = time.perf_counter()
    hist = C.train(s, ds, net, tr, epochs=args.epochs, batch=args.batch, lr=args.lr, lr_end=args.lr / 10)
    t_train = time.perf_counter() - t0
    fe = C.force_error(s, ds, net, hold)
    ev = C.evaluate(s, net, eval_seeds, t_end, every=args.every, t_attach=0.0)
    ds.buf.close()
    net.close()
    try:
        os.unlink(tune)
    except OSError:
        pass
    summ = {}
    for nm in ("plain", "closure"):
        summ[nm] = {
            "pk_max_rel_err": np.mean([e[nm]["pk_max_rel_err"] for e in ev], axis=0).tolist(),
            "pk_mean_rel_err": np.mean([e[nm]["pk_mean_rel_err"] for e in ev], axis=0).tolist(),
            "time_s": float(np.mean([e[nm]["time_s"] for e in ev]))}
    t_fine = float(np.mean([e["fine_time_s"] for e in ev]))
    worst = max(max(summ["closure"]["pk_max_rel_err"]), 0.0)
    return {"model": "two-field preheating (headline model), conformal", "n_fine": nf, "n_coarse": nc,
            "t_eval": t_end, "train_seeds": len(train_seeds), "eval_seeds": len(eval_seeds),
            "samples": ds.count, "heldout_samples": int(n_hold), "epochs": args.epochs,
            "loss_first_last": [hist[0], hist[-1]], "heldout_force_err": list(map(float, fe)),
            "pk_bins": "width 2pi/L up to half the coarse Nyquist wavenumber, fields phi and chi",
            "plain": summ["plain"], "closure": summ["closure"], "fine_time_s": t_fine,
            "speedup_closure_vs_fine": t_fine / summ["closure"]["time_s"],
            "speedup_plain_vs_fine": t_fine / summ["plain"]["time_s"],
            "target": "closure P(k) within 1% of the filtered fine run at >= 10x lower time to solution",
            "target_met": bool(worst <= 0.01 and t_fine / summ["closure"]["time_s"] >= 10.0),
            "data_gen_s": t_gen, "train_s": t_train,
            "scale_note": f"{nf}^3 -> {nc}^3 with {len(train_seeds)} training and {len(eval_seeds)} held-out seeds "
                          "(the benchmark's 512^3 -> 128^3 with 64 + 16 seeds runs as --case closure)"}


ENSEMBLE_SIZES = [64] * 32 + [96] * 32 + [128] * 24 + [192] * 8


def ensemble_workload(L, steps, warmup=3, tune=True):
    """96 independent phi^4 runs of uneven sizes (32 x 64^3, 32 x 96^3, 24 x 128^3,
    8 x 192^3), L = 20, spectral, Yoshida-4, dt = dx/20, FP32-Kahan, advanced
    together in a CUDA graph per call: per kick the streamed separable passes
    of every size class (two runs per complex line) or, when the autotuner
    picks it, per-class batched cuFFT around one persistent pass."""
    base = L.make_config(64, nfld=1, length=20.0, laplacian=L.LAP_SPECTRAL, precision=L.FP32_KAHAN,
                         model=L.MODEL_PHI4, model_params=(1.0,))
    ens = L.Ensemble(base, ENSEMBLE_SIZES)
    seeds = list(range(5000, 5000 + len(ENSEMBLE_SIZES)))
    ens.init_vacuum(seeds, 1.0, 0.0, 3.0, amp=1e-8, kcut_frac=0.5)
    if tune:
        ens.autotune(os.environ.get("LAT_TUNE_CACHE"))
    dto = 1.0 / 20
    ens.symp(4, dto, warmup)
    ens.prepare_symp(4, dto, steps)
    ens.sync()
    l0 = ens.launch_count()
    ens.mark(0)
    ens.symp(4, dto, steps)
    ens.mark(1)
    ms = ens.mark_elapsed(0, 1)
    launches = ens.launch_count() - l0
    E = ens.energies()
    S, W = ens.spectrum(len(ENSEMBLE_SIZES) - 1, 64)
    sites = sum(n ** 3 for n in ENSEMBLE_SIZES)
    out = {"runs": len(ENSEMBLE_SIZES), "sizes": "32x64^3 + 32x96^3 + 24x128^3 + 8x192^3", "steps": steps,
           "ms_per_step": ms / steps, "runs_per_s_1000_steps": len(ENSEMBLE_SIZES) / (ms / steps * 1000 * 1e-3),
           "site_updates_per_s": sites * steps / (ms * 1e-3), "tuning": ens.tuning(), "gpu_launches": launches,
           "spectral_path": "streamed separable passes (pairs of runs)" if ens.sep_streamed() else "cuFFT per class",
           "energy_finite": bool(np.all(np.isfinite(E))), "spectrum_bins_nonzero": int(np.count_nonzero(W))}
    ens.close()
    return out


def fd_workloads(L, hbm):
    """Site-updates/s and HBM fraction of the FD kick+drift passes."""
    res = {}
    # plain method: one field, phi^4, 64^3, L = 20, 7-point, leapfrog, dt = dx/10, FP64
    n = 64
    c = L.make_config(n, nfld=1, length=20.0, laplacian=L.LAP_FD7, precision=L.FP64, model=L.MODEL_PHI4)
    g = L.Lattice(c)
    g.init_vacuum(1000, [1.0], [0.0], [3.0], amp=1e-8, kcut_frac=0.5)
    g.autotune(os.environ.get("LAT_TUNE_CACHE"))
    dt = 20.0 / n / 10
    g.symp(2, dt, 10)
    g.prepare_symp(2, dt, 2000)  # graph built outside the timed region
    g.sync()
    g.mark(0)
    g.symp(2, dt, 2000)
    g.mark(1)
    ms = g.mark_elapsed(0, 1)
    res["phi4_64cube_fd7_fp64_leapfrog"] = {"steps": 2000, "ms_per_step": ms / 2000,
                                            "value": n ** 3 * 2000 / (ms * 1e-3), "unit": UNIT,
                                            "note": "whole 2000-step run, one symp2 call replayed as a CUDA graph"}
    g.close()
    # bubble collision with GW sourcing: 512^3, L = 128, 27-point, leapfrog, dt = dx/10, FP32 + Kahan
    n = 512
    g = L.Lattice(bubble_config(L, n))
    init_bubbles(g, n)
    g.autotune(os.environ.get("LAT_TUNE_CACHE"))
    dt = 0.25 / 10
    g.symp(2, dt, 3)
    K = 100  # one symp2 call; its leading and trailing half drifts are timed with it
    g.prepare_symp(2, dt, K)
    g.sync()
    g.mark(0)
    g.symp(2, dt, K)
    g.mark(1)
    ms = g.mark_elapsed(0, 1)
    g.timing(True)
    g.timing_reset()
    g.symp(2, dt, 5)
    g.sync()
    tkd, nkd = g.timing_read(L.K_KICKDRIFT)
    g.timing(False)
    bytes_kd = 120 * n ** 3  # phi (Kahan) 24 B + 6 u_ij and 6 pi_ij read+write 96 B
    ach = bytes_kd / (tkd / nkd * 1e-3) / 1e9 if nkd else None
    res["bubbles_512cube_fd27_gw_fp32"] = {"steps": K, "ms_per_step": ms / K, "value": n ** 3 * K / (ms * 1e-3),
                                           "tuning": g.tuning(),
                                           "unit": UNIT, "kickdrift_avg_us": 1e3 * tkd / max(nkd, 1),
                                           "kickdrift_achieved_gbs": ach,
                                           "kickdrift_frac": ach / hbm if ach else None,
                                           "algorithmic_bytes_per_site": 120}
    S, W = g.gw_spectrum(256)
    res["bubbles_512cube_fd27_gw_fp32"]["gw_spectrum_bins_nonzero"] = int(np.count_nonzero(W))
    g.close()
    return res


def bubble_config(L, n):
    """Bubble collision with GW sourcing: L = n/4, 27-point, DEFROST split, FP32 + Kahan."""
    return L.make_config(n, nfld=1, length=n / 4.0, laplacian=L.LAP_FD27, precision=L.FP32_KAHAN,
                         split_order=L.SPLIT_DEFROST, model=L.MODEL_DOUBLE_WELL, model_params=(0.01,), gw=True,
                         gw_coupling=2.0)


def init_bubbles(g, n):
    ln = n / 4.0
    g.init_bubbles([[0.34375 * ln, 0.5 * ln, 0.5 * ln], [0.65625 * ln, 0.5 * ln, 0.5 * ln]], 0.09375 * ln,
                   math.sqrt(2.0))


def run_conv_case(L, args, local):
    """The closure network's forward convolutions alone on an --n^3 lattice (default 128)."""
    net = L.Net(device=local, seed=11)
    out = conv_roofline(L, net, args.n or 128, reps=max(args.steps, 1))
    print(json.dumps({"metric": "closure forward convolutions, tensor FLOP/s", "case": "conv", **out}))
    return 0


def run_ensemble_case(L, args):
    """The batched uneven-size ensemble alone: 96 runs x --steps Yoshida-4 steps."""
    res = ensemble_workload(L, args.steps, args.warmup)
    print(json.dumps({"metric": "ensemble runs/s (96 uneven runs of 1000 Yoshida-4 steps, FP32-Kahan)",
                      "value": res["runs_per_s_1000_steps"], "unit": "runs/s", "case": "ensemble", **res}))
    return 0


def run_fd_case(L, args, local):
    """The FD bubble workload alone at side --n (used for profiling captures)."""
    n = args.n or 256
    c = bubble_config(L, n)
    c.device = local
    g = L.Lattice(c)
    init_bubbles(g, n)
    if not args.no_autotune:
        g.autotune(os.environ.get("LAT_TUNE_CACHE"))
    dt = 0.25 / 10
    g.symp(2, dt, args.warmup)
    g.prepare_symp(2, dt, args.steps)  # graph built outside the timed region
    g.sync()
    l0 = g.launch_count()
    g.mark(0)
    g.symp(2, dt, args.steps)
    g.mark(1)
    ms = g.mark_elapsed(0, 1)
    print(json.dumps({"metric": f"site-updates/s @{n}^3 FD27 bubbles + GW, leapfrog, FP32-Kahan", "tuning": g.tuning(),
                      "value": n ** 3 * args.steps / (ms * 1e-3), "unit": UNIT, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": ms / args.steps,
                      "gpu_launches": g.launch_count() - l0}))
    g.close()
    return 0


CONV_FLOPS_PER_SITE = {  # algorithmic tensor FLOPs per site (real channels: 4 -> 32 -> 32 -> 2)
    "conv1": 27 * 4 * 32 * 2,
    "conv2": 27 * 32 * 32 * 2,
    "conv3": 27 * 32 * 2 * 2,
}


def conv_roofline(L, net, n, reps=10):
    """Per-layer device time of the forward pass on an n^3 lattice and the
    algorithmic tensor FLOP rate against the measured dense BF16 peak."""
    ms = net.time_forward((n, n, n), reps)
    pk, kind = peaks()
    peak = float(pk.get("bf16_tflops", 1900.0))
    N = n ** 3
    out = {"lattice": n, "pack_ms": ms[0]}
    for i, name in enumerate(("conv1", "conv2", "conv3")):
        t = ms[i + 1] * 1e-3
        out[name] = {"ms": ms[i + 1], "tflops": N * CONV_FLOPS_PER_SITE[name] / t / 1e12}
    tot = sum(ms[1:]) * 1e-3
    ach = N * sum(CONV_FLOPS_PER_SITE.values()) / tot / 1e12
    out["roofline"] = {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                       "peak_kind": kind + " dense bf16 (cuBLAS burst)",
                       "note": "algorithmic FLOPs (the 4-channel input and the 2 outputs unpadded); conv1 "
                               "(4 padded to 8 -> 32) and conv2 (32->32) on tcgen05.mma with TMEM accumulators "
                               "when nx % 64 == 0, conv3 (32->2) weights-stationary on mma.sync; BF16 in, "
                               "FP32 accumulate"}
    return out


def closure_scenario(args, name):
    """Setup, time window and attach time of a closure scenario."""
    import importlib as _il
    C = _il.import_module("lattice-dev_gb300.closure")
    L = _il.import_module("lattice-dev_gb300")
    if name == "preheating":
        # the two-field preheating model from vacuum fluctuations, expanding, conformal units
        s = C.Setup(n_fine=args.n_fine, n_coarse=args.n or 64, tune_cache=os.environ.get("LAT_TUNE_CACHE"))
        return C, s, args.t_start, args.t_end, args.t_start
    # UV-rich fluctuations (<dphi^2> ~ 0.08) in Minkowski: the unresolved modes act on the
    # resolved ones through a mean-field force
    nf = args.n_fine
    s = C.Setup(n_fine=nf, n_coarse=args.n or nf // 4, length=nf / 8.0, background=L.BG_MINKOWSKI,
                kcut_frac=1.0, amp=0.01, units=L.UNITS_PROGRAM)
    return C, s, 0.5, 8.0, 0.0


def run_closure_case(L, args, local):
    """Learned closure: fine runs -> training data -> training -> held-out evaluation.

    Fine lattice args.n_fine^3 filtered to the coarse lattice (sharp-k), same
    box.  Prints one JSON line with the data, training and evaluation figures."""
    C, s, t0w, t1w, t_attach = closure_scenario(args, args.scenario)
    train_seeds = list(range(100, 100 + args.train_seeds))
    eval_seeds = list(range(900, 900 + args.eval_seeds))
    t0 = time.perf_counter()
    ds = C.generate(s, train_seeds, t0w, t1w, args.snapshots)
    t_gen = time.perf_counter() - t0
    net = L.Net(device=local, seed=11)
    norm = C.fit_norm(s, ds, net)
    n_hold = max(1, ds.count // 10)
    order = np.random.default_rng(0).permutation(ds.count)
    hold, tr = order[:n_hold], order[n_hold:]
    fe0 = C.force_error(s, ds, net, hold)
    t0 = time.perf_counter()
    hist = C.train(s, ds, net, tr, epochs=args.epochs, batch=args.batch, lr=args.lr, lr_end=args.lr / 10)
    t_train = time.perf_counter() - t0
    fe1 = C.force_error(s, ds, net, hold)
    shape = (s.n_coarse,) * 3
    t0 = time.perf_counter()
    for _ in range(5):
        net.train_step(ds.buf, s.stride, tr[:args.batch], shape, 1e-12)
    t_step = (time.perf_counter() - t0) / 5
    ev = C.evaluate(s, net, eval_seeds, t1w, every=args.every, t_attach=t_attach)
    ds.buf.close()
    summary = {}
    for nm in ("plain", "closure"):
        summary[nm] = {
            "pk_max_rel_err": np.mean([e[nm]["pk_max_rel_err"] for e in ev], axis=0).tolist(),
            "pk_mean_rel_err": np.mean([e[nm]["pk_mean_rel_err"] for e in ev], axis=0).tolist(),
            "time_s": float(np.mean([e[nm]["time_s"] for e in ev]))}
    t_fine = float(np.mean([e["fine_time_s"] for e in ev]))
    rl = conv_roofline(L, net, 128)
    print(json.dumps({
        "metric": "learned closure: P(k) error vs the filtered fine run, and time to solution",
        "case": "closure", "scenario": args.scenario, "n_fine": s.n_fine, "n_coarse": s.n_coarse,
        "length": s.length, "background": "conformal" if s.background == L.BG_CONFORMAL else "minkowski",
        "ic": {"amp": s.amp, "kcut_frac": s.kcut_frac}, "units": "conformal" if s.units else "program",
        "train_seeds": len(train_seeds), "eval_seeds": len(eval_seeds), "samples": ds.count,
        "t_window": [t0w, t1w], "t_eval": t1w, "t_attach": t_attach, "every": args.every,
        "pk_bins": "width 2pi/L up to half the coarse Nyquist wavenumber",
        "data_gen_s": t_gen, "train_s": t_train, "train_step_ms": 1e3 * t_step, "batch": args.batch,
        "epochs": args.epochs, "loss_first_last": [hist[0], hist[-1]],
        "norm": [list(map(float, v)) for v in norm],
        "heldout_force_err_untrained": list(map(float, fe0)), "heldout_force_err_trained": list(map(float, fe1)),
        "eval": ev, "summary": summary, "fine_time_s": t_fine,
        "speedup_closure_vs_fine": t_fine / summary["closure"]["time_s"],
        "speedup_plain_vs_fine": t_fine / summary["plain"]["time_s"],
        "conv_forward_128cube": rl}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-sub", type=int, default=10)
    ap.add_argument("--e2e-reps", type=int, default=5)
    ap.add_argument("--acc-steps", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--cpu-steps", type=int, default=24)
    ap.add_argument("--sustained-steps", type=int, default=1000,
                    help="steps of the extra long timed region reported under 'sustained' (0: skip)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fd", action="store_true")
    ap.add_argument("--no-closure", action="store_true")
    ap.add_argument("--closure-n-fine", type=int, default=256)
    ap.add_argument("--closure-train-seeds", type=int, default=4)
    ap.add_argument("--closure-eval-seeds", type=int, default=2)
    ap.add_argument("--quick", action="store_true", help="headline number only")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--spectral-impl", default="auto", choices=["auto", "cufft", "separable"])
    ap.add_argument("--n", type=int, default=None,
                    help="lattice side: headline 256 (other sides for profiling), fd-bubbles 256, closure coarse 64")
    ap.add_argument("--case", default="headline", choices=["headline", "fd-bubbles", "closure", "ensemble", "conv"],
                    help="fd-bubbles: the 27-point bubble-collision workload with GW sourcing at side --n; "
                         "closure: learned subgrid closure, fine --n-fine^3 filtered to --n^3")
    ap.add_argument("--n-fine", type=int, default=256)
    ap.add_argument("--scenario", default="preheating", choices=["preheating", "hartree"],
                    help="closure: two-field preheating from vacuum (expanding), or UV-rich fluctuations (Minkowski)")
    ap.add_argument("--train-seeds", type=int, default=8)
    ap.add_argument("--eval-seeds", type=int, default=2)
    ap.add_argument("--t-start", type=float, default=40.0)
    ap.add_argument("--t-end", type=float, default=120.0)
    ap.add_argument("--snapshots", type=int, default=17)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--every", type=int, default=3, help="closure: kicks per network evaluation")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
