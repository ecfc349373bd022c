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


def workload_config(L, precision, n=N_SIDE):
    return L.make_config(n, nfld=2, length=10 * math.pi, laplacian=L.LAP_SPECTRAL, background=L.BG_CONFORMAL,
                         precision=precision, model=L.MODEL_PHI4_G2, model_params=(1.0, 2.0))


def init_state(obj, seed):
    obj.init_vacuum(seed, [1.0, 0.0], [0.0, 0.0], [3.0, 2.0], amp=1e-8, kcut_frac=0.5)
    obj.set_scale_factor(1.0, 0.0)  # a(0) = 1, then ysclp from the Friedmann constraint
    obj.calc_metric()


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
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
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
def cpu_rate(steps_budget_s=20.0, max_steps=None, n=N_SIDE):
    """Times the CPU restatement (FP64, OpenMP on all host cores) on Yoshida-4
    steps of the same workload; returns (site-updates/s, cores, steps)."""
    import py_oracle
    L = importlib.import_module("lattice-dev_gb300")
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    c = workload_config(L, L.FP64, n)
    o = py_oracle.Oracle(c)
    init_state(o, 1000)
    dt = c.len / n / 20
    o.symp(4, dt, 1)  # warm-up (first-touch, FFT twiddles)
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
    rate, cores, done, el = cpu_rate(steps_budget_s=budget, max_steps=max(args.steps, 1))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT,
        "n_gpus": ws, "steps": done, "warmup": 1, "ms_per_step": 1e3 * el / done, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded vacuum fluctuations)",
        "config": {"workload": "two-field preheating 256^3, L=10pi, spectral, Yoshida-4, conformal, dt=dx/20",
                   "global_batch": N_SIDE ** 3, "seq_len": 1, "parallelism": "replicas"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{done} Yoshida-4 steps of the 256^3 workload after 1 warm-up step "
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
    c = workload_config(L, L.FP32_KAHAN)
    c.device = local
    g = L.Lattice(c)
    n = N_SIDE
    N = n ** 3
    dt = c.len / n / 20
    init_state(g, 1000 + rank)

    # warm-up
    g.symp(4, dt, W)
    g.sync()

    # timed region: exactly K Yoshida-4 steps in one symp4(dt, K) call
    sampler = ClockSampler(local)
    sampler.start()
    barrier(pg)
    g.sync()
    l0 = g.launch_count()
    g.mark(0)
    g.symp(4, dt, K)
    g.mark(1)
    g.sync()
    barrier(pg)
    ms = g.mark_elapsed(0, 1)
    launches = g.launch_count() - l0
    clocks = sampler.stop()
    ms = max_over_ranks(pg, ms)
    value = ws * N * K / (ms * 1e-3)

    extra = {}
    if rank == 0 and not args.quick:
        extra = diagnostics(L, g, args, dt, ms / K)
    g.close()

    if rank != 0:
        return 0
    pk, pk_kind = peaks()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (Kahan-compensated drifts, f64 reductions)",
        "data": "synthetic (seeded vacuum fluctuations, 1e-8/(2w_k) spectrum)",
        "config": {"workload": "two-field preheating 256^3, L=10pi, spectral, Yoshida-4, conformal, dt=dx/20",
                   "global_batch": N * ws, "seq_len": 1, "parallelism": f"replicas x{ws}",
                   "l2": "inputs larger than L2 (state 403 MB + spectra 270 MB per replica)"},
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
             L.K_FFT_R2C: "cufft_r2c", L.K_FFT_C2R: "cufft_c2r", L.K_OTHER: "other"}
    for k, nm in names.items():
        t, nl = g.timing_read(k)
        if nl:
            cls[nm] = {"ms": t, "launches": nl, "avg_us": 1e3 * t / nl}
    g.timing(False)
    tot = sum(v["ms"] for v in cls.values()) or 1.0
    for v in cls.values():
        v["share"] = v["ms"] / tot
    out["kernel_classes"] = cls
    # algorithmic bytes per launch of the engine kernels (2 fields)
    bytes_per = {"kickdrift": 2 * 28 * N, "kmul": 2 * 2 * 8 * (n // 2 + 1) * n * n,
                 "drift": 2 * 20 * N}
    own = {k: v for k, v in cls.items() if k in bytes_per}
    if own:
        dom = max(own, key=lambda k: own[k]["ms"])
        avg_s = own[dom]["avg_us"] * 1e-6
        ach = bytes_per[dom] / avg_s / 1e9
        out["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm, "unit": "GB/s",
                           "frac": ach / hbm, "traffic": None,
                           "algorithmic_bytes_per_launch": bytes_per[dom]}
    # whole step against the fused byte model (264.4 B per site-update)
    step_bytes = 3 * (2 * (2 * 4 * N + 2 * 8 * (n // 2 + 1) * n * n) + 2 * 28 * N)
    out["step_roofline"] = {"bytes_per_step": step_bytes, "achieved_gbs": step_bytes / (ms_step * 1e-3) / 1e9,
                            "frac": step_bytes / (ms_step * 1e-3) / 1e9 / hbm,
                            "model": "3 x (2 FFT r2c+c2r I/O + 28 B/site/field fused kick-drift)"}
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
        # ---- accuracy of FP32-Kahan against the FP64 GPU run from the same IC
        steps_acc = args.acc_steps
        c32 = workload_config(L, L.FP32_KAHAN)
        a32 = L.Lattice(c32)
        b64 = g64
        for obj in (a32, b64):
            init_state(obj, 4242)
        e0 = b64.energies()
        a32.symp(4, dt, steps_acc)
        b64.symp(4, dt, steps_acc)
        e32, e64 = a32.energies(), b64.energies()
        nb = 128
        acc = {"steps": steps_acc}
        for f in (0, 1):
            S32, _ = a32.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, nb)
            S64, _ = b64.spectrum(L.SPEC_FLD, f, L.SPEC_WEIGHTED, nb)
            live = np.arange(nb) >= 1
            rel = np.abs(S32[live] - S64[live]) / np.maximum(np.abs(S64[live]), 1e-300)
            acc[f"pk_field{f}_max_rel_err"] = float(np.max(rel[: n // 4]))
        acc["a_rel_err"] = abs(e32[L.E_A] - e64[L.E_A]) / e64[L.E_A]
        acc["friedmann_residual_fp32"] = float(e32[L.E_RESIDUAL])
        acc["friedmann_residual_fp64"] = float(e64[L.E_RESIDUAL])
        acc["friedmann_residual_initial"] = float(e0[L.E_RESIDUAL])
        out["accuracy_vs_fp64_gpu"] = acc
        a32.close()
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
    L.host_free(hf)
    L.host_free(hp)
    out["e2e"] = {"value": N * sub * reps / el, "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes,
                  "d2h_bytes_per_step": 2 * nbytes + 8 * L.NENERGY,
                  "step": f"lat_upload + lat_symp(4, dt, {sub}) + lat_energies + lat_download "
                          "(FP64 Fortran-layout pinned host arrays)"}
    # ---- CPU restatement on the host cores
    if not args.no_cpu:
        rate, cores, done, el = cpu_rate(steps_budget_s=args.cpu_budget, max_steps=args.cpu_steps)
        out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": f"{done} Yoshida-4 steps of the same 256^3 workload in FP64 "
                                         f"({el:.1f} s) after 1 warm-up step; CPU restatement of the "
                                         "Fortran reference, OpenMP"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-sub", type=int, default=10)
    ap.add_argument("--e2e-reps", type=int, default=5)
    ap.add_argument("--acc-steps", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--quick", action="store_true", help="headline number only")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
