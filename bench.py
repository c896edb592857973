"""Benchmark: lognormal shell maps per second at nside 2048 (40 shells, lmax 4096).

One step = one call of ``glass_gb300.generate`` producing 40 correlated
lognormal shell maps (HEALPix nside 2048, lmax 4096, float32 maps, complex64
alm) from their Gaussian angular power spectra: iternorm, Philox variates,
correlated alm, tensor-core Legendre contraction, ring FFTs and the fused
lognormal transform.  Synthetic spectra: C_l^ii = A_i (l+1)^-1.3 with A_i
log-uniform in [1e-3, 1e-1], correlation exp(-|i-j|/3), shifts uniform in
[0.5, 3], all from seed 0.

Printed JSON (one line, rank 0):
  value  -- shell-maps/s with spectra and maps resident on the device,
  e2e    -- the same through the public API from host (numpy) spectra to host
            (numpy) maps, copies inside the timed region (the median of 7
            calls; every call's time and the mean are in the line too),
  plain  -- the FP64 drop-in form on the same workload, and the fast form's
            relative RMS map error against it,
  roofline -- the Legendre contraction's algorithmic TF32 rate against the
            measured TF32 peak, with its DRAM bytes per launch,
  gpu_launches / clocks / cpu_baseline -- this library's launches in the
            timed region, SM clocks sampled during it, the CPU port's rate,
  serving -- p50/p99 latency and shell-maps/s of the serving workload: a
            Poisson stream of 2000 requests (nside in {128, 256, 512, 1024},
            lmax = 2 nside, 3-20 lognormal shells each) at 70% of the
            measured capacity, continuous batching within a 120 GB HBM
            budget; beside it the FP64 form without batching on a sample.

``--impl reference`` times the CPU restatement of the reference's path
(oracle/: GLASS glue + FP64 ring SHT with all host threads) on a bounded
sample of the same workload.  Multi-GPU (torchrun): replicas only -- every
rank runs the full workload; value = shells of all ranks / max time.
"""

from __future__ import annotations

import argparse
import json
import os
import pathlib
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "shell-maps/sec and pixels/sec at nside 2048 vs plain FP64 GPU @1e-6; p50/p99 latency"
UNIT = "shell-maps/s"
PASSES = 3  # tensor-core products per Legendre term (A_hi B_lo, A_lo B_hi, A_hi B_hi)
WORKLOAD = dict(workload="40-shell lognormal field generation, nside 2048, lmax 4096", nshell=40, nside=2048,
                lmax=4096)


def spectra_powerlaw13(nshell: int, lmax: int, seed: int = 0):
    rng = np.random.default_rng(seed)
    amp = 10 ** rng.uniform(-3, -1, nshell)
    lam = rng.uniform(0.5, 3.0, nshell)
    ell = np.arange(lmax + 1)
    auto = [a * (ell + 1.0) ** -1.3 for a in amp]
    gls = [np.exp(-abs(i - j) / 3.0) * np.sqrt(auto[i] * auto[j])
           for i in range(nshell) for j in range(i, -1, -1)]
    return gls, lam


def spectra_damped12(nshell: int, lmax: int, seed: int = 0):
    """Request spectra of the serving workload: A_i (l+1)^-1.2 e^{-(l/800)^2},
    A_i log-uniform in [1e-3, 1e-1], correlation exp(-|i-j|/1.5), shifts
    uniform in [0.5, 2]."""
    rng = np.random.default_rng(seed)
    amp = 10 ** rng.uniform(-3, -1, nshell)
    lam = rng.uniform(0.5, 2.0, nshell)
    ell = np.arange(lmax + 1)
    auto = [a * (ell + 1.0) ** -1.2 * np.exp(-((ell / 800.0) ** 2)) for a in amp]
    gls = [np.exp(-abs(i - j) / 1.5) * np.sqrt(auto[i] * auto[j])
           for i in range(nshell) for j in range(i, -1, -1)]
    return gls, lam


def _serving_requests(n: int, seed: int):
    """Requests of the serving workload: nside uniform over {128, 256, 512,
    1024}, lmax = 2 nside, 3-20 shells, per-request spectra seed."""
    from glass_gb300 import serving

    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        nside = int(rng.choice([128, 256, 512, 1024]))
        nshell = int(rng.integers(3, 21))
        gls, lam = spectra_damped12(nshell, 2 * nside, seed=seed * 100003 + i)
        reqs.append(serving.Request(gls=gls, nside=nside, shifts=[float(x) for x in lam], seed=1000 + i))
    return reqs


def _serve(reqs, rate: float | None, srv) -> dict:
    """Serve `reqs` arriving as a Poisson stream of `rate` requests/s (all at
    once when rate is None) on server `srv`; finished maps are dropped as
    they complete."""
    import torch

    form, batching = srv.form, srv.batching
    gaps = np.random.default_rng(7).exponential(1.0 / rate, len(reqs)) if rate else np.zeros(len(reqs))
    t0 = time.perf_counter() + 0.05
    arrivals = t0 + np.cumsum(gaps)
    for r, t in zip(reqs, arrivals):
        r.arrival = float(t)
        r.maps, r.finished, r.admitted = [], None, None

    def feeder():
        for r in reqs:
            dt = r.arrival - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            srv.submit(r)

    th = threading.Thread(target=feeder, daemon=True)
    th.start()
    done = 0
    while done < len(reqs):
        srv.step()
        while srv.finished:
            r = srv.finished.pop()
            r.maps = []  # the client has taken the maps
            done += 1
        if not srv.active:
            time.sleep(0.0002)
    th.join()
    torch.cuda.synchronize()
    lat = np.array([r.latency for r in reqs])
    shells = sum(r.nshell for r in reqs)
    span = max(r.finished for r in reqs) - min(r.arrival for r in reqs)
    return {"requests": len(reqs), "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
            "shell_maps_per_s": shells / span, "span_s": span,
            "arrival_rate_per_s": rate, "form": form, "batching": batching}


def run_serving(args) -> dict:
    """Serving workload on one long-running server: a closed warm-up batch
    (plans, fast tables, captured launch graphs), a closed calibration batch
    for the capacity, then a Poisson arrival stream at 70% of it; the FP64
    form without batching on a smaller sample for comparison."""
    from glass_gb300 import serving

    out = {}
    for form, batching, n, ncal in (("fast", True, args.serving, min(200, args.serving)),
                                    ("plain", False, args.serving_plain, min(20, args.serving_plain))):
        if n <= 0:
            continue
        srv = serving.Server(hbm_budget=120 << 30, form=form, batching=batching)
        _serve(_serving_requests(ncal, seed=17), None, srv)  # warm-up
        cal = _serve(_serving_requests(ncal, seed=91), None, srv)
        cap = cal["requests"] / cal["span_s"]
        res = _serve(_serving_requests(n, seed=3), 0.7 * cap, srv)
        res["capacity_req_per_s"] = cap
        res["launch_graphs"] = bool(getattr(srv, "graphs", False))
        out[f"{form}{'_batched' if batching else '_unbatched'}"] = res
        del srv
    return out


def run_shells10(steps: int = 3) -> dict:
    """10 correlated lognormal shells at nside 512 / lmax 1024
    (spectra A_i (l+1)^-1.2 e^{-(l/800)^2}, correlation e^{-|i-j|/1.5},
    shifts in [0.5, 2], from seed 0), device-resident.  Plain FP64 and fast
    forms timed with CUDA events (best of `steps`), the fast form's error per
    shell against the FP64 form (accuracy_report), and the spin-2 shear of
    the summed convergence (from_convergence, discretized) with its
    synthesis in both forms: times and the fast shear's error against FP64."""
    import torch

    import glass_gb300 as g

    nshell, nside, lmax = 10, 512, 1024
    gls_np, lam = spectra_damped12(nshell, lmax, seed=0)
    gls = [torch.as_tensor(c, device="cuda") for c in gls_np]
    fields = [g.grf.Lognormal(float(x)) for x in lam]
    out = {"workload": "10-shell lognormal field generation, nside 512, lmax 1024", "nshell": nshell,
           "nside": nside, "lmax": lmax}
    stream = torch.cuda.current_stream()
    for form in ("plain", "fast"):
        maps = list(g.generate(fields, gls, nside, rng=g.rng.Generator(42), form=form))  # warm-up
        best = None
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            maps = list(g.generate(fields, gls, nside, rng=g.rng.Generator(42), form=form))
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[form] = {"ms_per_step": best, "shell_maps_per_s": nshell / (best / 1e3)}
    out["fast_speedup"] = out["plain"]["ms_per_step"] / out["fast"]["ms_per_step"]
    rep = g.accuracy_report(fields, gls_np, nside, seed=42)
    out["fast_error_per_shell"] = rep
    out["fast_rel_rms_max"] = max(r["rms_rel"] for r in rep)
    kappa = torch.stack(maps).double().mean(dim=0)  # summed convergence (mean of the shells)
    shear = {"discretized": True, "lmax": 3 * nside - 1,
             "note": "analysis of kappa (map2alm, 3 iterations) in FP64 in both forms; the form is the synthesis'"}
    gam = {}
    for form in ("plain", "fast"):
        g.from_convergence(kappa, shear=True, form=form)  # warm-up (plans, spin tables, pixel windows)
        torch.cuda.synchronize()
        a = time.perf_counter()
        (gam[form],) = g.from_convergence(kappa, shear=True, form=form)
        torch.cuda.synchronize()
        shear[form] = {"ms": (time.perf_counter() - a) * 1e3}
    # the spin-2 synthesis alone (the shear's alm from one analysis), both forms
    lmx = 3 * nside - 1
    alm = g.healpix.analysis(kappa.reshape(1, -1), lmx, 3)[0]
    zero = torch.zeros_like(alm)
    for form in ("plain", "fast"):
        g.healpix.alm2map_spin([alm, zero], nside, 2, lmx, form=form)
        torch.cuda.synchronize()
        a = time.perf_counter()
        g.healpix.alm2map_spin([alm, zero], nside, 2, lmx, form=form)
        torch.cuda.synchronize()
        shear[form]["spin2_synthesis_ms"] = (time.perf_counter() - a) * 1e3
    d = gam["fast"].to(torch.complex128) - gam["plain"]
    shear["fast_vs_plain"] = {
        "rms_rel": float(torch.sqrt(torch.mean(d.abs() ** 2)) / torch.sqrt(torch.mean(gam["plain"].abs() ** 2))),
        "max_rel": float(d.abs().max() / gam["plain"].abs().max()),
        "max_abs": float(d.abs().max())}
    shear["finite"] = bool(torch.isfinite(gam["fast"]).all())
    out["shear"] = shear
    return out


def run_shells60(nshell: int = 60, nside: int = 4096, lmax: int = 8192) -> dict:
    """60 lognormal shells at nside 4096 / lmax 8192 (the 40-shell benchmark's
    spectra, seed 5) streamed through the fast form in groups of shells (as
    many as a 48 GB workspace allows), each shell consumed as it comes: its
    lognormal map added into the cumulative convergence (mean of the shells)
    and, for the first two, Poisson galaxy counts (5 per pixel) drawn from it
    as float32 and as float64 -- the counts must agree bit for bit, whichever
    form produced the delta values.  Then the spin-2 shear of the cumulative
    convergence (from_convergence, lmax 8192, FP64 form).  Device-resident;
    the nside-2048 plans are dropped first (their P_lm table would not leave
    room for this plan's 137 GB seed table)."""
    import torch

    import glass_gb300 as g
    from glass_gb300 import _lib

    _lib.clear_plans()
    torch.cuda.empty_cache()
    gls_np, lam = spectra_powerlaw13(nshell, lmax, seed=5)
    gls = [torch.as_tensor(c, device="cuda") for c in gls_np]
    fields = [g.grf.Lognormal(float(x)) for x in lam]
    npix = 12 * nside * nside
    out = {"workload": f"{nshell}-shell lognormal field generation streamed in groups, nside {nside}, lmax {lmax}",
           "nshell": nshell, "nside": nside, "lmax": lmax}
    a = time.perf_counter()
    next(iter(g.generate(fields[:1], gls[:1], nside, rng=g.rng.Generator(1), form="fast")))
    torch.cuda.synchronize()
    out["setup_s"] = time.perf_counter() - a  # plan, seeds, FFT tables, autotuning
    plan = _lib.get_plan(nside, lmax)
    out["plm_table"] = plan.has_plm_table
    out["plan_gb"] = plan.bytes / 1e9
    ngal = 5.0 * npix / g.points.ARCMIN2_SPHERE
    kappa = torch.zeros(npix, dtype=torch.float64, device="cuda")
    same, stream = [], torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    _lib.timing_enable(True)
    _lib.timing_reset()
    e0.record(stream)
    t_counts = 0.0
    for t, m in enumerate(g.generate(fields, gls, nside, rng=g.rng.Generator(42), form="fast")):
        kappa.add_(m, alpha=1.0 / nshell)
        if t < 2:
            c0 = torch.cuda.Event(enable_timing=True)
            c1 = torch.cuda.Event(enable_timing=True)
            c0.record(stream)
            n32 = g.points.counts_from_delta(ngal, m, rng=g.rng.Generator(7 + t))
            c1.record(stream)
            n64 = g.points.counts_from_delta(ngal, m.double(), rng=g.rng.Generator(7 + t))
            torch.cuda.synchronize()
            t_counts += c0.elapsed_time(c1)
            same.append(bool(torch.equal(n32, n64)))
            del n32, n64
        del m
    e1.record(stream)
    torch.cuda.synchronize()
    fast_kernels = {k: _lib.kernel_time(k) for k in ("k_leg_tc", "k_pack_b", "k_transpose32", "k_ring32",
                                                       "k_ring32_blu", "k_ring32_blug", "k_alm_correlate",
                                                       "k_iternorm", "k_refine", "k_poisson_counts")}
    _lib.timing_enable(False)
    ms = e0.elapsed_time(e1) - t_counts
    out["fast"] = {"ms": ms, "shell_maps_per_s": nshell / (ms / 1e3), "pixels_per_s": nshell * npix / (ms / 1e3),
                   "note": "includes the FP64 counts of two shells' float64 copies",
                   "kernel_ms_launches": fast_kernels}
    out["counts"] = {"bit_exact_f32_vs_f64_delta": all(same), "pixels_per_s": npix / (t_counts / 2 / 1e3),
                     "mean_per_pixel": 5.0}
    a = time.perf_counter()
    _lib.timing_enable(True)
    _lib.timing_reset()
    (gamma,) = g.from_convergence(kappa, lmax=lmax, shear=True)
    torch.cuda.synchronize()
    names = ("k_leg_ana", "k_leg_syn", "k_leg_syn_spin", "k_ring_ana", "k_ring_syn", "k_residual", "k_almxfl")
    kms = {k: _lib.kernel_time(k)[0] for k in names}
    _lib.timing_enable(False)
    out["shear"] = {"s": time.perf_counter() - a, "form": "plain FP64 (map2alm iter 3 + spin-2 synthesis)",
                    "lmax": lmax, "discretized": True, "finite": bool(torch.isfinite(gamma).all()),
                    "kernel_ms": kms}
    del gamma, kappa
    _lib.clear_plans()
    torch.cuda.empty_cache()
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
                for n, v in zip(names, r[3:7]):
                    if v.lower() in ("active", "1", "yes"):
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def tf32_peak_tflops(peaks: dict) -> tuple[float, str]:
    """Dense TF32 tensor peak: the tcgen05 kind::tf32 rate measured by
    ``bench.py --peaks`` (kept in profiles/peaks_tf32_fp64.json), else half
    the measured dense bf16 rate (same tensor pipe, tf32 at half the bf16
    rate)."""
    p = ROOT / "profiles" / "peaks_tf32_fp64.json"
    if p.exists():
        return float(json.loads(p.read_text())["tf32_tflops"]), "tf32 tcgen05 loop (of measured)"
    bf = peaks.get("bf16_tflops", 1900.0)
    tag = "of measured" if "fallback" not in peaks else "of fallback"
    return bf / 2.0, f"tf32 = bf16_tflops/2 ({tag})"


def measure_compute_peaks() -> dict:
    """TF32 tensor, FP32 and FP64 FMA rates of this GPU (the denominators the
    copy and bf16 GEMM figures do not give), with CUDA events, best of 5."""
    import ctypes

    import torch

    from glass_gb300 import _lib

    lib = _lib.lib()
    st = torch.cuda.current_stream()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    err = torch.zeros(1, dtype=torch.int32, device="cuda")

    def best(launch, reps=5):
        launch()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            launch()
            e1.record(st)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return min(ts)

    sp = ctypes.c_void_p(st.cuda_stream)
    iters = 40_000
    t = best(lambda: _lib.check(lib.glg_peak_tf32(sms, iters, ctypes.c_void_p(err.data_ptr()), sp), "glg_peak_tf32"))
    if int(err.item()) != 0:
        raise RuntimeError("glg_peak_tf32: a completion wait ran out")
    tf32 = sms * iters * 2.0 * 128 * 256 * 8 / t / 1e12
    out = {"tf32_tflops": round(tf32, 1), "tf32_how": f"{sms} CTAs x {iters} tcgen05.mma kind::tf32 M128 N256 K8"}
    for name, dt, dtype, it in (("fp32", torch.float32, _lib.GLG_F32, 16384), ("fp64", torch.float64, _lib.GLG_F64, 2048)):
        blocks = sms * 8
        sink = torch.zeros(blocks, dtype=dt, device="cuda")
        t = best(lambda: _lib.check(lib.glg_peak_fma(dtype, blocks, it, ctypes.c_void_p(sink.data_ptr()), sp),
                                    "glg_peak_fma"))
        out[f"{name}_tflops"] = round(blocks * 256 * it * 16.0 / t / 1e12, 2)
    out["fma_how"] = f"{sms * 8} blocks x 256 threads x 8 chains of FMA (2 flop each)"
    out["gpu_name"] = torch.cuda.get_device_name(0)
    return out


# ------------------------------------------------------------------- ours


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's time (all ranks receive it); `ms` itself at N = 1."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world: int, nshell: int, ms_step: float) -> float:
    """Whole-job throughput: every rank runs the full workload (replicas)."""
    return world * nshell / (ms_step / 1e3)


def run_ours(args, rank: int, world: int) -> dict | None:
    import torch

    import glass_gb300 as g
    from glass_gb300 import _lib

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    nshell, nside, lmax = args.nshell, args.nside, args.lmax
    gls_np, lam = spectra_powerlaw13(nshell, lmax)
    gls_dev = [torch.as_tensor(c, device=dev) for c in gls_np]
    ell = np.arange(lmax + 1)
    shell_variances = [np.sum((2 * ell + 1) * gls_np[k * (k + 1) // 2]) / (4 * np.pi) for k in range(nshell)]
    fields = [g.grf.Lognormal(float(x)) for x in lam]
    npix = 12 * nside * nside

    def step_device(form="fast"):
        out = list(g.generate(fields, gls_dev, nside, rng=g.rng.Generator(42), form=form))
        return out

    # warm-up (plan tables, seeds, allocator)
    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    _lib.timing_reset()
    launches0 = _lib.launch_count()
    stream = torch.cuda.current_stream()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(args.steps):
            step_device()
        t1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = max_over_ranks(t0.elapsed_time(t1), world, dev)
    launches = _lib.launch_count() - launches0
    ms_step = ms / args.steps
    value = job_value(world, nshell, ms_step)

    # per-kernel timing of the dominant kernel (one extra step, events per launch)
    _lib.timing_enable(True)
    _lib.timing_reset()
    step_device()
    torch.cuda.synchronize()
    kt = {k: _lib.kernel_time(k) for k in ("k_leg_tc", "k_pack_b", "k_transpose32", "k_ring32",
                                           "k_ring32_blu", "k_alm_correlate", "k_iternorm",
                                           "k_refine", "k_cls2cov", "k_cltovar")}
    _lib.timing_enable(False)
    leg_ms, leg_n = kt["k_leg_tc"]
    nalm = (lmax + 1) * (lmax + 2) // 2
    flops = 4.0 * nalm * 2 * nside * nshell  # algorithmic, dense (Legendre contraction)
    peaks = measured_peaks()
    peak_tf, peak_note = tf32_peak_tflops(peaks)
    achieved = flops / (leg_ms / max(leg_n, 1) / 1e3) / 1e12 if leg_ms > 0 else None
    # DRAM bytes of one full-size k_leg_tc launch (40 maps, nside 2048, lmax
    # 4096, P_lm table path), scaled from the ncu capture of the same launch
    # at nside 512 / lmax 1024 (bench.py --ncu-case leg: 2.052 GB read, 0.644
    # GB written) by the table size (138.0 / 2.20 GB) for the reads and by
    # the Legendre sums' size (10.74 / 0.671 GB) for the writes
    # (profiles/leg_tc_plm_40maps_nside512.md)
    table = g.healpix.get_plan(nside, lmax).has_plm_table
    traffic = (2.052e9 * 138.0 / 2.20 + 0.644e9 * 10.74 / 0.671) if table and (nshell, nside, lmax) == (
        40, 2048, 4096) else None
    roofline = {"bound": "tensor", "kernel": "k_leg_tc", "achieved": achieved, "peak": peak_tf,
                "unit": "TFLOP/s", "frac": (achieved / peak_tf) if achieved else None,
                "traffic": traffic, "traffic_unit": "bytes per launch", "peak_note": peak_note, "passes": PASSES,
                "issued_frac": (PASSES * achieved / peak_tf) if achieved else None,
                "algorithmic_flops_per_launch": flops}
    # the same figure against the measured bf16 GEMM rate halved (the
    # tensor pipe's tf32 rate is half its bf16 rate)
    bf_half = peaks.get("bf16_tflops", 1900.0) / 2.0
    if traffic:  # the same launch against the measured copy bandwidth
        gbs = traffic / (leg_ms / max(leg_n, 1) / 1e3) / 1e9
        roofline["hbm"] = {"achieved": gbs, "peak": peaks.get("hbm_gbs", 6800.0), "unit": "GB/s",
                           "frac": gbs / peaks.get("hbm_gbs", 6800.0), "traffic_note": "scaled from nside 512"}
    roofline["vs_bf16_half"] = {"peak": bf_half, "frac": (achieved / bf_half) if achieved else None,
                                "issued_frac": (PASSES * achieved / bf_half) if achieved else None,
                                "note": "of measured" if "fallback" not in peaks else "of fallback"}
    if rank != 0:
        return None

    # plain FP64 form on the same workload, and the fast form's error against it
    plain = {}
    if args.plain_steps > 0:
        torch.cuda.synchronize()
        a = time.perf_counter()
        pm = step_device("plain")
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - a
        fm = step_device("fast")
        errs, maxs = [], []
        for x, y in zip(fm, pm):
            d = x.double() - y
            errs.append(float(torch.sqrt(torch.mean(d * d)) / torch.sqrt(torch.mean(y * y))))
            maxs.append(float(d.abs().max() / y.abs().max()))
        plain = {"value": nshell / plain_s, "unit": UNIT, "ms_per_step": plain_s * 1e3,
                 "fast_vs_plain_rel_rms_max": max(errs), "fast_vs_plain_rel_rms_median": float(np.median(errs)),
                 "fast_vs_plain_rel_rms_per_shell": errs, "fast_vs_plain_rel_max_per_shell": maxs,
                 "shell_variances": [float(v) for v in shell_variances],
                 "speedup": (nshell / plain_s) and value / (nshell / plain_s)}
        del pm, fm
        torch.cuda.empty_cache()  # the FP64 form's buffers: room for the host-output workspace

    # galaxy counts and positions on the benchmark's fast maps (n = 5 per
    # pixel on average): Poisson counts of 4 shells, positions of one
    points = {}
    if args.points:
        maps = step_device()
        ngal = 5.0 * npix / g.points.ARCMIN2_SPHERE
        gen = g.rng.Generator(7)
        g.points.counts_from_delta(ngal, maps[0], rng=gen)  # warm-up
        for _ in g.points.positions_from_delta(ngal, maps[1], batch=100_000_000, rng=gen):
            pass  # warm-up: the batches' buffers come from the allocator's cache in the timed pass
        torch.cuda.synchronize()
        _lib.timing_enable(True)
        _lib.timing_reset()
        for t in range(4):
            g.points.counts_from_delta(ngal, maps[t], rng=gen)
        torch.cuda.synchronize()
        c_ms, _ = _lib.kernel_time("k_poisson_counts")
        a = time.perf_counter()
        ngal_out = sum(int(c) for _, _, c in g.points.positions_from_delta(ngal, maps[1], batch=100_000_000, rng=gen))
        torch.cuda.synchronize()
        p_wall = time.perf_counter() - a
        p_ms, _ = _lib.kernel_time("k_positions")
        _lib.timing_enable(False)
        points = {"mean_per_pixel": 5.0, "counts_pixels_per_s": 4 * npix / (c_ms / 1e3),
                  "positions_galaxies": ngal_out, "positions_kernel_galaxies_per_s": ngal_out / (p_ms / 1e3),
                  "positions_from_delta_galaxies_per_s": ngal_out / p_wall}
        del maps
        torch.cuda.empty_cache()  # the 100M-galaxy batches' blocks: e2e starts from the same state either way

    # end to end: numpy spectra in, numpy maps out, through the public API
    e2e = {}
    if args.e2e_steps > 0:
        # one untimed call sizes the pinned host buffers; every timed call
        # hands its numpy maps to the caller, who drops them before the next
        maps = list(g.generate(fields, gls_np, nside, rng=g.rng.Generator(42), form="fast"))
        d2h = int(sum(m.nbytes for m in maps))
        del maps
        torch.cuda.synchronize()
        a = time.perf_counter()
        calls = []
        for _ in range(args.e2e_steps):
            c = time.perf_counter()
            maps = list(g.generate(fields, gls_np, nside, rng=g.rng.Generator(42), form="fast"))
            del maps
            calls.append((time.perf_counter() - c) * 1e3)
        torch.cuda.synchronize()
        mean_s = (time.perf_counter() - a) / args.e2e_steps
        # the median call: a call copies 8 GB into host memory, and on a host
        # shared with other jobs an occasional call's copies run 1.2-5x slower
        # (the synthesis alone measured 54.5 ms in most calls, 66-274 ms in a
        # few, with the same pinned buffer); every call and the mean are kept
        e_s = float(np.median(calls)) / 1e3
        e2e = {"value": nshell / e_s, "unit": UNIT, "ms_per_step": e_s * 1e3, "statistic": "median call",
               "ms_per_call": calls, "mean_ms_per_call": mean_s * 1e3, "value_of_mean": nshell / mean_s,
               "h2d_bytes_per_step": int(sum(c.nbytes for c in gls_np)),
               "d2h_bytes_per_step": d2h}

    serving = run_serving(args) if (args.serving > 0 or args.serving_plain > 0) else None
    shells10 = run_shells10() if args.shells10 else None
    shells60 = None
    if args.shells60:
        try:
            shells60 = run_shells60()
        except Exception as exc:  # noqa: BLE001 - recorded, the headline stands
            shells60 = {"error": f"{type(exc).__name__}: {exc}"}
    cpu = cpu_baseline(args) if args.cpu_baseline else None
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 maps / 3xtf32 contraction / f64 recurrence seeds",
        "data": "synthetic spectra (seeded), Philox variates",
        "config": dict(WORKLOAD, form="fast", l2="inputs/outputs larger than L2 (maps 8 GB/step)",
                       parallelism="replicas" if world > 1 else "1 gpu"),
        "pixels_per_sec": value * npix, "e2e": e2e, "plain_fp64": plain, "roofline": roofline, "points": points,
        "kernel_ms_per_step": {k: v[0] for k, v in kt.items()},
        "kernel_launches_per_step": {k: v[1] for k, v in kt.items()}, "gpu_launches": launches,
        "clocks": clk.summary(), "cpu_baseline": cpu, "serving": serving,
        "shells10_nside512": shells10, "shells60_nside4096": shells60,
    }
    return res


def cpu_baseline(args) -> dict:
    """The oracle (GLASS glue + FP64 ring SHT, all host threads) on a 1-shell
    sample of the same workload; value in shell-maps/s."""
    import oracle
    import oracle.fields as of
    import oracle.rng as orng

    gls, lam = spectra_powerlaw13(args.nshell, args.lmax)
    sample = max(1, args.cpu_shells)
    a = time.perf_counter()
    it = of.generate_lognormal(gls, args.nside, list(lam), ncorr=None,
                               z_of_shell=lambda t, s: orng.complex_normals(42, t, 0, s))
    for _ in range(sample):
        next(it)
    dt = time.perf_counter() - a
    return {"value": sample / dt, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{sample} of {args.nshell} shells at nside {args.nside}, lmax {args.lmax} "
                      "(iternorm of all shells, Philox variates, C Legendre sums, numpy ring FFTs)"}


# -------------------------------------------------------------- reference


def run_reference(args, rank: int, world: int) -> dict | None:
    if rank != 0:
        return None
    args.cpu_shells = 1
    vals = []
    for _ in range(max(args.warmup, 0)):
        pass  # the oracle has no device state to warm
    for _ in range(args.steps):
        r = cpu_baseline(args)
        vals.append(r["value"])
    v = float(np.median(vals))
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic spectra (seeded)",
            "config": dict(WORKLOAD, form="cpu port"), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": r["cores"], "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def ncu_case(which: str) -> None:
    """Small profiling cases (no JSON).  "sht": two fast `generate` calls of 8
    lognormal shells of the serving spectra at nside 1024, lmax 2048 (the
    Legendre sums, 0.54 GB, exceed L2); profilers capture the first call.
    "alm": the correlated alm of the benchmark's 40 shells at lmax 4096 in the
    fast form (2.7 GB written, no transform), twice.  "leg": two fast
    syntheses of 40 maps at nside 512, lmax 1024 (the contraction's P_lm
    table 2.2 GB and its Legendre sums 0.67 GB exceed L2; about 4 GB on the
    device)."""
    import torch

    import glass_gb300 as g

    if which == "leg":
        from glass_gb300 import healpix as hp

        lmax = 1024
        rng = np.random.default_rng(5)
        n = (lmax + 1) * (lmax + 2) // 2
        alm = torch.as_tensor(rng.standard_normal((40, n)) + 1j * rng.standard_normal((40, n)),
                              dtype=torch.complex64, device="cuda")
        for _ in range(2):
            maps = hp.synth(alm, 512, lmax, form="fast")
            torch.cuda.synchronize()
        print("ncu case done", float(maps.abs().max()))
        return

    if which == "alm":
        from glass_gb300 import fields

        gls = [torch.as_tensor(c, device="cuda") for c in spectra_powerlaw13(40, 4096)[0]]
        b = fields._FieldBatcher(gls, 2048, None, g.rng.Generator(42), "fast")
        for _ in range(2):
            alm = b.alm(0, 40)
            torch.cuda.synchronize()
        print("ncu case done", float(alm.abs().max()))
        return
    gls, lam = spectra_damped12(8, 2048, seed=1)
    gls = [torch.as_tensor(c, device="cuda") for c in gls]
    fields = [g.grf.Lognormal(float(x)) for x in lam]
    for _ in range(2):
        maps = list(g.generate(fields, gls, 1024, rng=g.rng.Generator(42), form="fast"))
        torch.cuda.synchronize()
    print("ncu case done", float(maps[0].abs().max()))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--nshell", type=int, default=40)
    ap.add_argument("--nside", type=int, default=2048)
    ap.add_argument("--lmax", type=int, default=4096)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=7)
    ap.add_argument("--cpu-shells", type=int, default=1)
    ap.add_argument("--serving", type=int, default=2000, help="requests of the serving workload (0: off)")
    ap.add_argument("--serving-plain", type=int, default=60,
                    help="requests of the FP64 unbatched serving comparison (0: off)")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-shells10", dest="shells10", action="store_false",
                    help="skip the 10-shell nside-512 record")
    ap.add_argument("--no-shells60", dest="shells60", action="store_false",
                    help="skip the 60-shell nside-4096 streamed record")
    ap.add_argument("--no-points", dest="points", action="store_false",
                    help="skip the galaxy counts / positions aside")
    ap.add_argument("--ncu-case", nargs="?", const="sht", choices=["sht", "alm", "leg"],
                    help="run a small profiling case and exit")
    ap.add_argument("--peaks", action="store_true", help="measure the TF32 / FP32 / FP64 peak rates and exit")
    args = ap.parse_args()
    if args.ncu_case:
        ncu_case(args.ncu_case)
        return
    if args.peaks:
        print(json.dumps(measure_compute_peaks()))
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist

        dist.init_process_group("nccl")
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
