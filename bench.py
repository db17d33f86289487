#!/usr/bin/env python
"""Benchmark: SO(3) forward+inverse transform pairs per second at l_max = 255.

Workload (default): a batch of complex SO(3) functions at l_max = 255 (512^3
Euler grid each, complex64 samples; synthetic seeded coefficients
F ~ N(0,1)(l+1)^-1.5), transformed with the tensor-core split-BF16 path
(FFTSO3_PREC_TC_BF16X3, stable Wigner-d recursion).  One step = inverse of the
whole batch (coefficients -> grids) + forward of the whole batch
(grids -> coefficients); value = functions / step time.  The library runs
on one GPU (no sharding, no collectives): launched with more than one rank,
rank 0 prints a line saying so and no GPU work is done.

Also reported: the plain FP64 GPU path on the same l_max (pairs/s), the
accuracy of the tensor-core path against FP64, the end-to-end rate through the
host-buffer C-ABI calls, the roofline of the dominant kernel (stage timing
with CUDA events inside the library), and the CPU baseline: the oracle's
restatement of the reference algorithm timed on the host cores on a bounded
sample of beta slices.

--impl reference times only that CPU algorithm (all host threads) on the same
workload and prints its own JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "SO(3) fwd+inv transforms/s at l_max=255: TC split-BF16 vs FP64 at rel-err<=1e-6"
UNIT = "transform pairs/s"


def seeded_coeffs(l_max: int, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    l = np.concatenate([np.full((2 * x + 1) ** 2, x) for x in range(l_max + 1)])
    s = (l + 1.0) ** -1.5
    return rng.standard_normal(l.size) * s + 1j * rng.standard_normal(l.size) * s


def per_l_errors(a: np.ndarray, b: np.ndarray, l_max: int) -> tuple[float, float]:
    """rel_rms = ||a-b|| / ||b||; rel_max = max_l max_mn |a-b| / rms_mn |b| (per-l normalised)."""
    rms = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    mx = 0.0
    for l in range(l_max + 1):
        o0, o1 = l * (4 * l * l - 1) // 3, (l + 1) * (4 * (l + 1) ** 2 - 1) // 3
        d = np.abs(a[o0:o1] - b[o0:o1]).max()
        r = np.sqrt(np.mean(np.abs(b[o0:o1]) ** 2))
        mx = max(mx, float(d / r))
    return rms, mx


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9 and f[1].replace(".", "").isdigit():
                    rows.append(f)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        under = [s for s in sm if s > 0.5 * mx] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(under)), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())
                if any(r[3].replace(".", "").isdigit() for r in rows) else None}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def profiled_traffic(stage: str, l_max: int, batch: int):
    """DRAM bytes per launch of `stage` from the committed ncu capture figures
    (profiles/traffic.json: stage, l_max, batch, bytes per launch), scaled to
    this workload: by batch at the same l_max, and for the FFT stages (whose
    traffic is one read and one write of every sample) by batch * N^3 across l_max."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    found = [(r["l_max"], r["batch"], r["bytes_per_launch"]) for r in json.load(open(path))["captures"]
             if r["stage"] == stage]
    for L0, b0, byts in found:
        if L0 == l_max:
            return byts * batch / b0
    for L0, b0, byts in found:
        if stage.startswith("fft"):
            return byts * batch / b0 * ((l_max + 1) / (L0 + 1)) ** 3
    return None


# --------------------------------------------------------------- CPU legs

def cpu_sample(l_max: int, nslices: int | None = None, threads: int | None = None) -> dict:
    """Oracle (the reference algorithm restated, OpenMP over beta slices as the reference) on S beta slices
    spread evenly over [0, pi) -- k = stride/2 + i stride -- of one l_max forward and one inverse; pairs/s
    extrapolated to all 2B slices (every slice costs the same work)."""
    from oracle import oracle as O

    O.build()
    nth = threads or os.cpu_count() or 1
    O.set_num_threads(nth)
    N = 2 * (l_max + 1)
    S = max(1, min(N, nslices or nth))
    stride = N // S
    k0 = stride // 2
    rng = np.random.default_rng(0)
    F = seeded_coeffs(l_max, 0)
    slab = (rng.standard_normal((S, N, N)) + 1j * rng.standard_normal((S, N, N)))
    t0 = time.perf_counter()
    O.so3_forward_complex_strided(l_max, slab, k0, stride)
    t1 = time.perf_counter()
    O.so3_inverse_complex_strided(l_max, F, k0, stride, S)
    t2 = time.perf_counter()
    per_pair = ((t1 - t0) + (t2 - t1)) * N / S
    return {"value": 1.0 / per_pair, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"{S} of {N} beta slices (k = {k0} + {stride} i, spread over [0, pi)) of one l_max={l_max} "
                      f"complex forward and inverse (oracle restatement of fdcl_FFTSO3.cpp:659-763 / :498-531, "
                      f"OpenMP over slices, {nth} threads); pairs/s extrapolated x{N}/{S}",
            "seconds": t2 - t0}


def cpu_baselines(l_max: int) -> dict:
    """The CPU baseline at all host threads (the reported figure) and at one thread, as the reference's
    example4 times its transforms (example/example4.cpp:30,58)."""
    nth = os.cpu_count() or 1
    full = cpu_sample(l_max, nslices=2 * nth, threads=nth)
    one = cpu_sample(l_max, nslices=2, threads=1)
    full.pop("seconds", None)
    one.pop("seconds", None)
    full["single_thread"] = {"value": one["value"], "cores": 1, "sample": one["sample"]}
    return full


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    nth = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(args.l_max, nslices=nth)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_sample(args.l_max, nslices=nth))
    wall = time.perf_counter() - t0
    v = float(np.mean([x["value"] for x in vals]))
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": f"SO(3) complex forward+inverse, l_max={args.l_max}, batch={args.batch} functions per "
                               f"GPU ({2 * (args.l_max + 1)}^3 grid each); the reference's CPU algorithm (oracle port, "
                               "all host threads) timed on a bounded sample of beta slices of one function, pairs/s "
                               "extrapolated per function",
                   "l_max": args.l_max, "batch_per_gpu": args.batch, "precision": "f64 (CPU)"},
        "cpu_baseline": {k: vals[-1][k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- uneven batch

UNEVEN_METRIC = "SO(3) real fwd+inv transforms/s, 4096 functions, l_max~U{8..64}: TC batch vs FP64 per-function loop"


def uneven_lmax(n: int, seed: int = 3) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.integers(8, 65, size=n)


def main_uneven(args) -> None:
    """The batching workload: n real SO(3) functions with l_max drawn uniformly
    from {8..64}, FP32 samples, coefficients N(0,1)/(2l+1); one fftso3_batch
    (tensor-core buckets, CUDA graph).  Compared with a per-function launch loop
    of the plain FP64 path (one batch-1 FFTSO3_REAL FP64 plan per l_max)."""
    import torch

    from fftso3_gb300 import _lib
    from fftso3_gb300 import build as fbuild

    fbuild.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    n = args.functions
    lmax = uneven_lmax(n)
    t_create = time.perf_counter()
    bt = _lib.Batch(_lib.SO3_REAL, lmax, "tc_bf16x3", "reference", _lib.FLAG_GRAPH | _lib.FLAG_AUTOTUNE)
    t_create = time.perf_counter() - t_create
    G, Ctot = bt.grid_elems, bt.coeff_elems
    # seeded coefficients N(0,1)/(2l+1), generated on the device per function
    Lm = int(lmax.max())
    deg = torch.from_numpy(np.concatenate([np.full((2 * l + 1) ** 2, l) for l in range(Lm + 1)])).to(dev)
    scale = 1.0 / (2.0 * deg.double() + 1.0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(11)
    coef = torch.empty(Ctot, dtype=torch.float32, device=dev)
    for i in range(n):
        o0 = bt.coeff_offset(i)
        c = _lib.lib().fftso3_coeff_elems(_lib.SO3_REAL, int(lmax[i]))
        coef[o0:o0 + c] = (torch.randn(c, generator=gen, device=dev, dtype=torch.float64) * scale[:c]).float()
    grid = torch.empty(G, dtype=torch.float32, device=dev)
    bt.inverse(coef.data_ptr(), grid.data_ptr(), sp)      # band-limited FP32 samples
    grid_out = torch.empty_like(grid)
    coef_out = torch.empty_like(coef)
    torch.cuda.synchronize()
    bt.check()

    # accuracy on a sample of functions against the FP64 plain path on the same FP32 samples
    acc_rms, acc_idx = [], []
    plans64 = {}
    bt.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
    for i in np.linspace(0, n - 1, 8).astype(int):
        L = int(lmax[i])
        p = plans64.setdefault(L, _lib.Plan(_lib.SO3_REAL, L, 1, "fp64", "reference"))
        g0, c0 = bt.grid_offset(i), bt.coeff_offset(i)
        gi = grid[g0:g0 + p.grid_elems].double()
        ci = torch.empty(p.coeff_elems, dtype=torch.float64, device=dev)
        p.forward(gi.data_ptr(), ci.data_ptr(), sp)
        torch.cuda.synchronize()
        a = coef_out[c0:c0 + p.coeff_elems].double()
        acc_rms.append(float(torch.linalg.norm(a - ci) / torch.linalg.norm(ci)))
        acc_idx.append(int(i))
    bt.check()

    # ---- timed region (inputs resident; 10+ GB of samples >> L2)
    for _ in range(args.warmup):
        bt.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
        bt.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            bt.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
            bt.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    bt.check()
    clocks = clk.summary()
    value = n * 1000.0 / ms
    # one more step, eager with per-stage events, for the stage breakdown
    bt.set_timing(True)
    bt.stage_times(reset=True)
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    bt.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
    bt.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
    s1.record(stream)
    torch.cuda.synchronize()
    eager_ms = s0.elapsed_time(s1)
    st_all = bt.stage_times()
    per_bucket = []
    for k in range(bt.buckets):
        L, cnt = bt.bucket_info(k)
        t = bt.stage_times(bucket=k)
        per_bucket.append((sum(v for v, _ in t.values()), L, cnt, {a: round(v, 3) for a, (v, _) in t.items()}))
    bt.stage_times(reset=True)
    bt.set_timing(False)
    per_bucket.sort(reverse=True)
    stage_summary = {k: {"ms": v, "launches": c} for k, (v, c) in st_all.items()}
    launches = int(sum(c for _, c in st_all.values()))
    io_bytes = 2.0 * 4.0 * (G + Ctot)  # per pair: grid + coefficients read once and written once
    peaks = measured_peaks()

    # ---- baseline: per-function launch loop of the FP64 path (one FP64 plan per l_max)
    fp64 = None
    if not args.no_fp64:
        for L in sorted(set(int(x) for x in lmax)):
            plans64.setdefault(L, _lib.Plan(_lib.SO3_REAL, L, 1, "fp64", "reference"))
        g64 = grid.double()
        c64 = coef.double()
        go64 = torch.empty_like(g64)
        co64 = torch.empty_like(c64)
        goff = [bt.grid_offset(i) for i in range(n)]
        coff = [bt.coeff_offset(i) for i in range(n)]
        gp, cp, gop, cop = g64.data_ptr(), c64.data_ptr(), go64.data_ptr(), co64.data_ptr()

        def loop():
            for i in range(n):
                p = plans64[int(lmax[i])]
                p.inverse(cp + 8 * coff[i], gop + 8 * goff[i], sp)
                p.forward(gp + 8 * goff[i], cop + 8 * coff[i], sp)

        loop()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        loop()
        f1.record(stream)
        torch.cuda.synchronize()
        ms64 = f0.elapsed_time(f1)
        fp64 = {"value": n * 1000.0 / ms64, "unit": UNIT, "ms_per_step": ms64,
                "note": "per-function launch loop, FFTSO3_REAL FP64 plans (batch 1, one per l_max), float64 samples"}
        del g64, c64, go64, co64
    line = {
        "metric": UNEVEN_METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16x3 (split) / fp32 accumulate / fp32 FFT; fp32 samples",
        "data": "synthetic",
        "config": {"workload": f"{n} real SO(3) functions, l_max uniform in 8..64 (seed 3), coefficients "
                               "N(0,1)/(2l+1), FP32 samples; fftso3_batch, tensor-core buckets, CUDA graph, "
                               "autotuned",
                   "functions": n, "buckets": bt.buckets, "streams": bt.streams, "samples": int(G),
                   "coefficients": int(Ctot), "autotune": "FFT launch shapes per N, bucket streams",
                   "l2": "inputs larger than L2"},
        "io_gbs": io_bytes / (ms / 1000.0) / 1e9, "io_frac_of_hbm": io_bytes / (ms / 1000.0) / 1e9 / peaks["hbm_gbs"],
        "batch_create_s": t_create, "device_gb": bt.device_bytes / 1e9,
        "accuracy": {"rel_rms_vs_fp64_max": max(acc_rms), "functions": acc_idx},
        "fp64_loop": fp64, "speedup_vs_fp64_loop": value / fp64["value"] if fp64 else None,
        "clocks": clocks, "gpu_launches": launches * args.steps,
        "stages_eager_sum_ms": stage_summary, "eager_timed_step_ms": eager_ms,
        "top_buckets": [{"l_max": L, "functions": c, "ms": t, "stages": d} for t, L, c, d in per_bucket[:6]],
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- FP64 plain path

FP64_METRIC = "SO(3) FP64 fwd+inv transforms/s at l_max={L}: plain FP64 GPU path (complex and real)"


def main_fp64(args) -> None:
    """The plain FP64 GPU path (FFTSO3_PREC_FP64, reference recursion) on one function at
    l_max = 127 (256^3 grid), complex and real: transform pairs/s, HBM GB/s of the FFT passes
    and of the table generation (plan creation), FP64 rate of the beta-sum."""
    import torch

    from fftso3_gb300 import _lib
    from fftso3_gb300 import build as fbuild

    fbuild.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    L = args.fp64_l_max
    B, N = L + 1, 2 * (L + 1)
    C = B * (4 * B * B - 1) // 3
    out = {}
    for kind, name in ((_lib.SO3_COMPLEX, "complex"), (_lib.SO3_REAL, "real")):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p = _lib.Plan(kind, L, 1, "fp64", "reference")
        torch.cuda.synchronize()
        t_plan = time.perf_counter() - t0
        cplx = kind == _lib.SO3_COMPLEX
        dt = torch.complex128 if cplx else torch.float64
        rng = np.random.Generator(np.random.PCG64(5))
        l = np.concatenate([np.full((2 * x + 1) ** 2, x) for x in range(B)])
        F = rng.standard_normal(C) / (2 * l + 1)
        if cplx:
            F = F + 1j * rng.standard_normal(C) / (2 * l + 1)
        c = torch.from_numpy(F).to(dev)
        g = torch.empty(N ** 3, dtype=dt, device=dev)
        c2 = torch.empty_like(c)
        for _ in range(args.warmup):
            p.inverse(c.data_ptr(), g.data_ptr(), sp)
            p.forward(g.data_ptr(), c2.data_ptr(), sp)
        torch.cuda.synchronize()
        p.set_timing(True)
        p.stage_times(reset=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            p.inverse(c.data_ptr(), g.data_ptr(), sp)
            p.forward(g.data_ptr(), c2.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        st = p.stage_times(reset=True)
        p.set_timing(False)
        p.check()
        rel = float(torch.linalg.norm(c2 - c) / torch.linalg.norm(c))
        esz = 16 if cplx else 8
        grid_b = 16.0 * N ** 3  # complex128 work grid
        fft = {}
        for k in ("fft_rows", "fft_cols"):
            if k in st:
                t = st[k][0] / st[k][1] / 1000.0
                fft[k] = {"ms_per_launch": t * 1000.0, "gbs": 2 * grid_b / t / 1e9}
        table_bytes = 8.0 * sum((2 * m + 1) * (B - m) for m in range(B)) * N
        flops = 8.0 * B * C  # beta-sum per direction
        contr = {}
        for k in ("fp64_fwd_contract", "fp64_inv_contract"):
            if k in st:
                t = st[k][0] / st[k][1] / 1000.0
                contr[k] = {"ms_per_launch": t * 1000.0, "fp64_tflops": flops / t / 1e12}
        out[name] = {"pairs_per_s": 1000.0 / ms, "ms_per_pair": ms, "round_trip_rel_err": rel,
                     "fft": fft, "contraction": contr,
                     "table": {"plan_create_s": t_plan, "table_gb": table_bytes / 1e9,
                               "table_gbs_incl_setup": table_bytes / t_plan / 1e9},
                     "stages_ms": {k: v for k, (v, _) in st.items()}, "grid_elem_bytes": esz}
        del p, c, g, c2
        torch.cuda.empty_cache()
    line = {"metric": FP64_METRIC.format(L=L), "value": out["complex"]["pairs_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["complex"]["ms_per_pair"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"one SO(3) function, l_max={L} ({N}^3 grid), FP64, reference recursion; "
                                   "coefficients N(0,1)/(2l+1)"},
            "complex": out["complex"], "real": out["real"]}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- point evaluation

POINTS_METRIC = "SO(3) point evaluations/s at l_max={L}: inverse_transform(F, alpha, beta, gamma) at {n} rotations, FP64"
S2_POINTS_METRIC = "S^2 point evaluations/s at l_max={L}: inverse_transform(F, theta, phi) at {n} points, FP64"
FP64_NOMINAL_TFLOPS = 1.25  # GB300 FP64 (no FP64 figure among the measured peaks)


def main_points(args) -> None:
    """Batched point evaluation (fftso3_inverse_points, the reference's inverse_transform(F, alpha,
    beta, gamma) of fdcl_FFTSO3.cpp:498-531 at many rotations) of one complex function at l_max = 127
    (the size of the reference's own per-point timing), n seeded random rotations per call, FP64 with
    the reference recursion.  CPU baseline: the oracle's restatement of the same function, one point per
    host thread; the first points are also compared against the GPU values."""
    import torch
    from concurrent.futures import ThreadPoolExecutor

    from fftso3_gb300 import _lib
    from fftso3_gb300 import build as fbuild

    fbuild.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    s2 = args.points_kind == "s2"
    L, n = (args.s2_l_max if s2 else args.points_l_max), args.points
    B = L + 1
    rng = np.random.Generator(np.random.PCG64(11))
    if s2:
        C = B * B
        l = np.concatenate([np.full(2 * x + 1, x) for x in range(B)])
        F = (rng.standard_normal(C) + 1j * rng.standard_normal(C)) / (l + 1.0)
        plan = _lib.Plan(_lib.S2_COMPLEX, L, 1, "fp64", "reference")
        pts = np.ascontiguousarray(np.column_stack([rng.uniform(0.0, np.pi, n), rng.uniform(0.0, 2 * np.pi, n)]))
    else:
        C = B * (4 * B * B - 1) // 3
        F = seeded_coeffs(L, 0)
        plan = _lib.Plan(_lib.SO3_COMPLEX, L, 1, "fp64", "reference")
        pts = np.ascontiguousarray(np.column_stack([rng.uniform(-np.pi, np.pi, n), rng.uniform(0.0, np.pi, n),
                                                    rng.uniform(-np.pi, np.pi, n)]))
    c = torch.from_numpy(F).to(dev)
    out = np.empty(n, dtype=np.complex128)

    def call():
        plan.inverse_points(c.data_ptr(), 0, pts.ctypes.data_as(_lib._dp), n, out.ctypes.data, sp)

    for _ in range(args.warmup):
        call()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(args.steps):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) / args.steps
    ms = e0.elapsed_time(e1) / args.steps
    clocks = clk.summary()
    plan.check()
    value = n * 1000.0 / ms
    # algorithmic work per point: SO(3) the (2l+1) F d products, 6 FP64 flops per coefficient; S^2 the
    # F nP products, 4 flops per coefficient
    fpc = 4.0 if s2 else 6.0
    achieved = fpc * C * n / (ms / 1000.0) / 1e12
    roof = {"bound": "fp64", "unit": "TFLOP/s", "kernel": "s2_points_kernel" if s2 else "so3_points_kernel",
            "achieved": achieved, "peak": FP64_NOMINAL_TFLOPS, "frac": achieved / FP64_NOMINAL_TFLOPS,
            "peak_source": "nominal",
            "algorithmic": f"{int(fpc)} flops per coefficient per point (the recursion's flops not counted)",
            "traffic": None}
    cpu = None
    parity = None
    if not args.no_cpu:
        from oracle import oracle as O

        O.build()
        nth = os.cpu_count() or 1
        ns = min(n, 10 * nth)
        t0 = time.perf_counter()
        one = (lambda i: O.s2_inverse_complex_point(L, F, *pts[i])) if s2 else \
            (lambda i: O.so3_inverse_complex_point(L, F, *pts[i]))
        if s2:
            ns = min(n, 200 * nth)
        with ThreadPoolExecutor(max_workers=nth) as ex:
            ref = list(ex.map(one, range(ns)))
        dt = time.perf_counter() - t0
        ref = np.array(ref)
        parity = {"points": ns, "rel_err": float(np.linalg.norm(out[:ns] - ref) / np.linalg.norm(ref)),
                  "max_abs_err": float(np.abs(out[:ns] - ref).max())}
        src = ("fdcl_FFTS2.cpp:194-230 with its Legendre recursion :48-100" if s2 else
               "fdcl_FFTSO3.cpp:498-531 with its Wigner-d recursion :127-194")
        cpu = {"value": ns / dt, "unit": "points/s", "cores": nth, "kind": "port",
               "sample": f"the first {ns} of the {n} points, one point per host thread (oracle restatement of "
                         f"{src})", "seconds": dt}
    what = (f"one complex S^2 function, l_max={L} (C={C} coefficients, N(0,1)/(l+1)), {n} seeded random points "
            "per call, FP64, the reference's Legendre recursion" if s2 else
            f"one complex SO(3) function, l_max={L} (C={C} coefficients, N(0,1)(l+1)^-1.5), "
            f"{n} seeded random rotations per call, FP64, reference recursion")
    line = {"metric": (S2_POINTS_METRIC if s2 else POINTS_METRIC).format(L=L, n=n), "value": value,
            "unit": "points/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": what,
                       "l2": "coefficients (one 16-byte read per coefficient per point) stay in L2"},
            "e2e": {"value": n / wall, "unit": "points/s", "h2d_bytes_per_step": (16 if s2 else 24) * n,
                    "d2h_bytes_per_step": 16 * n},
            "gpu_launches": args.steps, "roofline": roof, "clocks": clocks, "cpu_baseline": cpu, "parity": parity}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- grid FFT stage

FFT_METRIC = "SO(3) grid FFT stage GB/s (grids <-> pencils, one launch per direction), N={N}, {nf} grids"


def main_fft(args) -> None:
    """The grid FFT stage alone (fftso3_grid_fft) on nf complex64 grids of N^3 samples:
    one step = the grids -> pencils launch and the pencils -> grids launch.  GB/s counts
    the algorithmic bytes (each sample read once and written once per launch)."""
    import torch

    from fftso3_gb300 import _lib
    from fftso3_gb300 import build as fbuild

    fbuild.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    N, nf = args.fft_n, args.batch
    gen = torch.Generator(device=dev).manual_seed(3)
    g = torch.randn((nf, N, N, N), dtype=torch.complex64, device=dev, generator=gen)
    pen = torch.empty_like(g)
    back = torch.empty_like(g)
    nws = _lib.grid_fft_workspace_bytes(N, nf)
    wbuf = torch.zeros(nws + 256, dtype=torch.uint8, device=dev)
    ws = wbuf.data_ptr() + (-wbuf.data_ptr()) % 256

    def step():
        _lib.grid_fft(N, nf, 1, False, g.data_ptr(), pen.data_ptr(), ws, sp)
        _lib.grid_fft(N, nf, -1, False, pen.data_ptr(), back.data_ptr(), ws, sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    _lib.grid_fft_check(ws, sp)
    ms = e0.elapsed_time(e1) / args.steps
    idx = (-torch.arange(N, device=dev)) % N
    rel = float(torch.linalg.vector_norm(back[0] - g[0][:, idx][:, :, idx] * (N * N)) /
                torch.linalg.vector_norm(g[0] * (N * N)))
    byts = 2 * 2 * 8.0 * nf * N ** 3  # two launches, each reads and writes every complex64 sample
    peaks = measured_peaks()
    gbs = byts / (ms / 1000.0) / 1e9
    line = {"metric": FFT_METRIC.format(N=N, nf=nf), "value": gbs, "unit": "GB/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (complex64)", "data": "synthetic",
            "config": {"workload": f"{nf} complex64 grids of {N}^3 samples (N(0,1)), forward then inverse direction",
                       "l2": f"inputs larger than L2 ({8.0 * nf * N ** 3 / 1e9:.1f} GB per array)"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": gbs / peaks["hbm_gbs"], "peak_source": peaks["source"],
                         "algorithmic": "one read + one write of every sample per launch"},
            "double_transform_rel_err": rel, "gpu_launches": 2 * args.steps,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- S^2 batch

S2_METRIC = "S2 real fwd+inv transforms/s, {b} signals at l_max={L}: TC split-BF16 vs FP64"


def main_s2(args) -> None:
    """512 real S^2 signals at l_max = 511 (1024 x 1024 grids, FP32 samples,
    coefficients N(0,1)/(l+1)) through one FFTS2_real tensor-core plan."""
    import torch

    from fftso3_gb300 import _lib
    from fftso3_gb300 import build as fbuild

    fbuild.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    L, b = args.s2_l_max, args.functions if args.functions != 4096 else 512
    B, N = L + 1, 2 * (L + 1)
    C = B * B
    plan = _lib.Plan(_lib.S2_REAL, L, b, "tc_bf16x3", "reference")
    deg = torch.from_numpy(np.concatenate([np.full(2 * l + 1, l) for l in range(B)])).to(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(21)
    coef = (torch.randn(b, C, generator=gen, device=dev, dtype=torch.float64) / (deg.double() + 1.0)).float()
    grid = torch.empty(b * N * N, dtype=torch.float32, device=dev)
    plan.inverse(coef.data_ptr(), grid.data_ptr(), sp)
    grid_out = torch.empty_like(grid)
    coef_out = torch.empty_like(coef)
    torch.cuda.synchronize()
    plan.check()

    # accuracy of signal 0 against the FP64 plan (same FP32-rounded coefficients and samples)
    p64 = _lib.Plan(_lib.S2_REAL, L, 1, "fp64", "reference")
    c0 = coef[0].double().contiguous()
    g64 = torch.empty(N * N, dtype=torch.float64, device=dev)
    p64.inverse(c0.data_ptr(), g64.data_ptr(), sp)
    F64 = torch.empty(C, dtype=torch.float64, device=dev)
    g0 = grid[:N * N].double().contiguous()
    p64.forward(g0.data_ptr(), F64.data_ptr(), sp)
    plan.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
    plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
    torch.cuda.synchronize()
    plan.check()
    acc = {"forward_rel_rms": float(torch.linalg.norm(coef_out[0].double() - F64) / torch.linalg.norm(F64)),
           "inverse_rel_rms": float(torch.linalg.norm(grid_out[:N * N].double() - g64) / torch.linalg.norm(g64)),
           "against": "FP64 plan (FFTS2_real, FP64) on signal 0"}
    # the same signal through the FP32 CUDA-core beta-sum (same FP32 FFT): separates GEMM and FFT error
    p32 = _lib.Plan(_lib.S2_REAL, L, 1, "fp32", "reference")
    c32 = torch.empty(C, dtype=torch.float32, device=dev)
    g32 = torch.empty(N * N, dtype=torch.float32, device=dev)
    p32.forward(grid.data_ptr(), c32.data_ptr(), sp)
    p32.inverse(coef.data_ptr(), g32.data_ptr(), sp)
    torch.cuda.synchronize()
    acc["fp32_cuda_core_forward_rel_rms"] = float(torch.linalg.norm(c32.double() - F64) / torch.linalg.norm(F64))
    acc["fp32_cuda_core_inverse_rel_rms"] = float(torch.linalg.norm(g32.double() - g64) / torch.linalg.norm(g64))
    del p32, c32, g32

    # FP64 path rate (batch 16, per signal)
    b64 = 16
    p64b = _lib.Plan(_lib.S2_REAL, L, b64, "fp64", "reference")
    cb = coef[:b64].double().contiguous()
    gb = torch.empty(b64 * N * N, dtype=torch.float64, device=dev)
    ob = torch.empty_like(cb)
    p64b.inverse(cb.data_ptr(), gb.data_ptr(), sp)
    p64b.forward(gb.data_ptr(), ob.data_ptr(), sp)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    f0.record(stream)
    p64b.inverse(cb.data_ptr(), gb.data_ptr(), sp)
    p64b.forward(gb.data_ptr(), ob.data_ptr(), sp)
    f1.record(stream)
    torch.cuda.synchronize()
    fp64 = {"value": b64 * 1000.0 / f0.elapsed_time(f1), "unit": UNIT, "batch": b64,
            "note": "plain FP64 GPU path (FFTS2_real, FP64), same l_max"}
    del p64b, cb, gb, ob

    for _ in range(args.warmup):
        plan.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
        plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            plan.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
            plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clocks = clk.summary()
    plan.set_timing(True)
    plan.stage_times(reset=True)
    plan.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
    plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
    torch.cuda.synchronize()
    stages = plan.stage_times(reset=True)
    plan.set_timing(False)
    plan.check()
    peaks = measured_peaks()
    flops = 4.0 * N * B * B * b  # useful flops per direction (pairs m, -m; re/im)
    gemm = {}
    for name in ("tc_gemm_fwd", "tc_gemm_inv"):
        if name in stages:
            t = stages[name][0] / stages[name][1] / 1000.0
            gemm[name] = {"ms": t * 1000.0, "tflops": flops / t / 1e12,
                          "frac_of_bf16": flops / t / 1e12 / peaks["bf16_tflops_sustained"]}
    fft_bytes = 4.0 * b * N * N + 8.0 * b * N * N  # real samples + complex pencils, one pass
    fft = {}
    for name in ("fft_rows",):
        if name in stages:
            t = stages[name][0] / stages[name][1] / 1000.0
            fft[name] = {"ms": t * 1000.0, "gbs": fft_bytes / t / 1e9, "frac_of_hbm": fft_bytes / t / 1e9 / peaks["hbm_gbs"]}
    value = b * 1000.0 / ms
    line = {
        "metric": S2_METRIC.format(b=b, L=L), "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16x3 (split) / fp32 accumulate / fp32 FFT; fp32 samples", "data": "synthetic",
        "config": {"workload": f"{b} real S^2 signals, l_max={L} ({N}x{N} grid, FP32 samples), coefficients "
                               "N(0,1)/(l+1); FFTS2_real tensor-core plan", "signals": b, "l_max": L,
                   "l2": "inputs larger than L2 (2 GB of samples)"},
        "accuracy": acc, "fp64_path": fp64, "speedup_vs_fp64_path": value / fp64["value"],
        "gemm": gemm, "fft": fft,
        "stages": {k: {"ms": v, "launches": c} for k, (v, c) in stages.items()},
        "gpu_launches": int(sum(c for _, c in stages.values())) * args.steps, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- GPU arm

def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--l-max", type=int, default=255)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp32", action="store_true", help="skip the FP32 CUDA-core beta-sum comparison")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 reference (profiling runs)")
    ap.add_argument("--workload", default="lmax255", choices=["lmax255", "uneven", "s2", "fp64", "fft", "points"],
                    help="lmax255: the headline SO(3) batch at one l_max (--l-max/--batch); uneven: the "
                         "mixed-bandwidth SO(3) batch; s2: the S^2 batch at l_max=511")
    ap.add_argument("--functions", type=int, default=4096, help="uneven workload: number of functions")
    ap.add_argument("--s2-l-max", type=int, default=511, help="s2 workload: l_max")
    ap.add_argument("--fp64-l-max", type=int, default=127, help="fp64 workload: l_max")
    ap.add_argument("--fft-n", type=int, default=512, help="fft workload: grid size N (64..512), --batch grids")
    ap.add_argument("--points", type=int, default=4096, help="points workload: rotations per call")
    ap.add_argument("--points-l-max", type=int, default=127, help="points workload: l_max (SO(3))")
    ap.add_argument("--points-kind", default="so3", choices=["so3", "s2"],
                    help="points workload: SO(3) rotations (--points-l-max) or S^2 points (--s2-l-max)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args)
        return
    if world > 1 or args.gpus > 1:
        # one GPU by design: no rank touches a GPU, rank 0 says why
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps({"metric": METRIC, "n_gpus": max(world, args.gpus), "impl": "gb300",
                              "unavailable": "single-GPU library: each transform runs on one GPU with no sharding "
                                             "or collectives; the headline is measured with --gpus 1"}),
                  flush=True)
        return
    if args.workload == "uneven":
        main_uneven(args)
        return
    if args.workload == "s2":
        main_s2(args)
        return
    if args.workload == "fp64":
        main_fp64(args)
        return
    if args.workload == "fft":
        main_fft(args)
        return
    if args.workload == "points":
        main_points(args)
        return

    import torch

    import fftso3_gb300 as fg
    from fftso3_gb300 import _lib
    from fftso3_gb300 import build as fbuild

    fbuild.build()
    rank = 0
    local = 0
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    L, b = args.l_max, args.batch
    N = 2 * (L + 1)
    C = fg.so3_ncoeff(L)

    def barrier():
        torch.cuda.synchronize()

    # ---- FP64 plain path: reference data for the accuracy check + its own rate
    F0 = seeded_coeffs(L, 1000 * rank)
    fp64 = None
    acc = {}
    if args.no_accuracy:
        args.no_fp64 = True
    p64 = None if args.no_accuracy else _lib.Plan(_lib.SO3_COMPLEX, L, 1, "fp64", "stable")
    c64 = torch.from_numpy(F0).to(dev)
    g64 = torch.empty(N ** 3, dtype=torch.complex128, device=dev)
    o64 = torch.empty_like(c64)
    if p64 is not None:
        p64.inverse(c64.data_ptr(), g64.data_ptr(), sp)
        p64.forward(g64.data_ptr(), o64.data_ptr(), sp)
    torch.cuda.synchronize()
    F0_fp64 = o64.cpu().numpy()  # FP64 forward of the FP64 synthesis
    g0_c64 = g64.to(torch.complex64)
    g0_ref = g64.cpu().numpy()
    if not args.no_fp64:
        reps = 2
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            p64.inverse(c64.data_ptr(), g64.data_ptr(), sp)
            p64.forward(g64.data_ptr(), o64.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        fp64 = {"value": 1000.0 / ms, "unit": UNIT, "ms_per_pair": ms, "batch": 1,
                "note": "plain FP64 GPU path (FFTSO3_PREC_FP64, stable recursion), same l_max"}
    del p64, g64, o64, c64
    torch.cuda.empty_cache()

    # ---- tensor-core plan
    plan = _lib.Plan(_lib.SO3_COMPLEX, L, b, "tc_bf16x3", "stable", _lib.FLAG_AUTOTUNE)
    Fb = np.concatenate([seeded_coeffs(L, 1000 * rank + i) for i in range(b)]).astype(np.complex64)
    coef = torch.from_numpy(Fb).to(dev)
    grid = torch.empty(b * N ** 3, dtype=torch.complex64, device=dev)
    plan.inverse(coef.data_ptr(), grid.data_ptr(), sp)  # synthetic band-limited inputs
    if not args.no_accuracy:
        grid[:N ** 3].copy_(g0_c64)                     # function 0: the FP64 synthesis
    coef_out = torch.empty_like(coef)
    grid_out = torch.empty_like(grid)
    torch.cuda.synchronize()
    plan.check()

    # accuracy vs FP64 (function 0), before the timed region
    coef0 = torch.from_numpy(F0.astype(np.complex64)).to(dev)
    coef_in = coef.clone()
    coef_in[:C].copy_(coef0)
    if not args.no_accuracy:
        plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
        plan.inverse(coef_in.data_ptr(), grid_out.data_ptr(), sp)
        torch.cuda.synchronize()
        plan.check()
        fr, fm = per_l_errors(coef_out[:C].cpu().numpy().astype(np.complex128), F0_fp64, L)
        gi = grid_out[:N ** 3].cpu().numpy().astype(np.complex128)
        ir = float(np.linalg.norm(gi - g0_ref) / np.linalg.norm(g0_ref))
        im = float(np.abs(gi - g0_ref).max() / np.sqrt(np.mean(np.abs(g0_ref) ** 2)))
        acc = {"forward_rel_rms": fr, "forward_rel_max_per_l": fm, "inverse_rel_rms": ir,
               "inverse_rel_max": im, "against": "FP64 GPU path (stable recursion) on the same function"}
        # one residual refinement step F += forward(f - inverse(F)) (FFTSO3_FLAG_REFINE), same function
        pr = _lib.Plan(_lib.SO3_COMPLEX, L, 1, "tc_bf16x3", "stable", _lib.FLAG_REFINE)
        cr = torch.empty(C, dtype=torch.complex64, device=dev)
        pr.forward(g0_c64.data_ptr(), cr.data_ptr(), sp)
        e0r, e1r = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0r.record(stream)
        pr.forward(g0_c64.data_ptr(), cr.data_ptr(), sp)
        e1r.record(stream)
        torch.cuda.synchronize()
        pr.check()
        rr, rm = per_l_errors(cr.cpu().numpy().astype(np.complex128), F0_fp64, L)
        acc["refined_forward_rel_rms"] = rr
        acc["refined_forward_rel_max_per_l"] = rm
        acc["refined_forward_ms_batch1"] = e0r.elapsed_time(e1r)
        del pr, cr
    del coef_in, coef0

    # ---- timed region: inputs resident in HBM (each grid 1 GB >> 129 MB L2)
    for _ in range(args.warmup):
        plan.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
        plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
    barrier()
    plan.set_timing(True)
    plan.stage_times(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            plan.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
            plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    stages = plan.stage_times(reset=True)
    plan.set_timing(False)
    plan.check()
    clocks = clk.summary()
    ms_max = ms
    value = b * 1000.0 / ms_max
    launches = int(sum(c for _, c in stages.values()))

    # ---- roofline of the dominant kernel
    peaks = measured_peaks()
    B = L + 1
    top = max(stages.items(), key=lambda kv: kv[1][0])
    name, (tot_ms, cnt) = top
    per_launch_s = tot_ms / cnt / 1000.0
    useful_flops = 8.0 * B * C * b            # complex beta-sum flops per direction for the batch
    grid_bytes = 8.0 * b * N ** 3             # one complex64 pass over the batch's grids
    if name.startswith("tc_gemm"):
        achieved = useful_flops / per_launch_s / 1e12
        peak = peaks["bf16_tflops_sustained"]
        roof = {"bound": "tensor", "unit": "TFLOP/s", "algorithmic": "8*B*C*batch useful flops per launch"}
    else:
        if name.startswith("fft") or name.startswith("tc_pack"):
            byts = 2 * grid_bytes  # one complex64 read and write of the batch's grids (FFT pass / transpose)
        else:
            byts = grid_bytes
        achieved = byts / per_launch_s / 1e9
        peak = peaks["hbm_gbs"]
        roof = {"bound": "hbm", "unit": "GB/s", "algorithmic": "bytes read + written per launch"}
    roof.update({"kernel": name, "achieved": achieved, "peak": peak, "frac": achieved / peak,
                 "peak_source": peaks["source"], "ms_per_launch": per_launch_s * 1000.0,
                 "traffic": profiled_traffic(name, L, b)})
    stage_summary = {k: {"ms_per_launch": v / c, "launches": c, "share": v / sum(x for x, _ in stages.values())}
                     for k, (v, c) in stages.items()}
    # ---- roofline of the whole step: the larger of its HBM floor (algorithmic bytes of every stage) and its
    # tensor floor (the issued split-BF16 MMA flops), against the measured step time
    Kp = (N + 63) // 64 * 64
    table_rows = sum((2 * m + 1) * (B - m) for m in range(B))  # rows l of all symmetry groups
    table_b = 3 * 2.0 * Kp * table_rows                        # three BF16 planes, read once per GEMM launch
    coef_b = 8.0 * b * C                                        # complex64 coefficients of the batch
    step_bytes = (2 * 2 * grid_bytes                            # FFT: two launches, one read + one write each
                  + 2 * (grid_bytes + table_b + coef_b)         # GEMMs: pencils + table + coefficients
                  + 2 * 2 * coef_b)                             # coefficient permutations
    hbm_floor_ms = step_bytes / (peaks["hbm_gbs"] * 1e9) * 1e3
    tensor_floor_ms = 2 * 6 * useful_flops / (peaks["bf16_tflops_sustained"] * 1e12) * 1e3
    floor_ms = max(hbm_floor_ms, tensor_floor_ms)
    step_roof = {"bound": "hbm" if hbm_floor_ms >= tensor_floor_ms else "tensor", "algorithmic_bytes": step_bytes,
                 "hbm_floor_ms": hbm_floor_ms, "tensor_floor_ms": tensor_floor_ms, "ms_per_step": ms_max,
                 "frac": floor_ms / ms_max, "peak_source": peaks["source"],
                 "note": "FFT 4 x grid bytes, GEMMs 2 x (pencils + BF16 table planes + coefficients), permutations "
                         "4 x coefficients; tensor floor = 6 issued BF16 products of the 8BC useful flops, both "
                         "directions"}

    # ---- end to end through the host-buffer C ABI (pinned host memory)
    e2e = None
    if not args.no_e2e:
        hg = torch.empty(b * N ** 3, dtype=torch.complex64, pin_memory=True)
        hg.copy_(grid)
        hc = torch.empty(b * C, dtype=torch.complex64, pin_memory=True)
        hc.copy_(coef)
        hco = torch.empty_like(hc, pin_memory=True)
        # the inverse writes the grid the forward then reads (one pinned grid buffer)
        plan.inverse_host(hc.data_ptr(), hg.data_ptr(), sp)
        plan.forward_host(hg.data_ptr(), hco.data_ptr(), sp)
        barrier()
        t0 = time.perf_counter()
        ksteps = args.steps  # the same step count as the device-timed region
        for _ in range(ksteps):
            plan.inverse_host(hc.data_ptr(), hg.data_ptr(), sp)
            plan.forward_host(hg.data_ptr(), hco.data_ptr(), sp)
        barrier()
        dt = (time.perf_counter() - t0) / ksteps
        e2e = {"value": b / dt, "unit": UNIT, "h2d_bytes_per_step": int(8 * b * C + 8 * b * N ** 3),
               "d2h_bytes_per_step": int(8 * b * N ** 3 + 8 * b * C), "steps": ksteps}
        del hg, hc, hco

    # ---- the FP32 form of the beta-sum (CUDA cores, FFTSO3_PREC_FP32) on the same batch
    fp32 = None
    plan.close()  # the tensor-core plan's tables and workspace make room for the FP32 plan
    del plan, grid_out, coef_out
    torch.cuda.empty_cache()
    if not args.no_fp32:
        p32 = _lib.Plan(_lib.SO3_COMPLEX, L, b, "fp32", "stable")
        g32 = torch.empty_like(grid)
        c32 = torch.empty_like(coef)
        p32.inverse(coef.data_ptr(), g32.data_ptr(), sp)
        p32.forward(grid.data_ptr(), c32.data_ptr(), sp)
        torch.cuda.synchronize()
        p32.check()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        p32.inverse(coef.data_ptr(), g32.data_ptr(), sp)
        p32.forward(grid.data_ptr(), c32.data_ptr(), sp)
        f1.record(stream)
        torch.cuda.synchronize()
        ms32 = f0.elapsed_time(f1)
        fp32 = {"value": b * 1000.0 / ms32, "unit": UNIT, "ms_per_step": ms32,
                "note": "FFTSO3_PREC_FP32: FP32 table and FMA accumulation on the CUDA cores, same batch"}
        if not args.no_accuracy:
            pa = _lib.Plan(_lib.SO3_COMPLEX, L, 1, "fp32", "stable")
            ca = torch.empty(C, dtype=torch.complex64, device=dev)
            pa.forward(g0_c64.data_ptr(), ca.data_ptr(), sp)
            torch.cuda.synchronize()
            fr32, fm32 = per_l_errors(ca.cpu().numpy().astype(np.complex128), F0_fp64, L)
            fp32.update({"forward_rel_rms": fr32, "forward_rel_max_per_l": fm32})
            del pa, ca
        del p32, g32, c32
        torch.cuda.empty_cache()

    # ---- the refined forward (FFTSO3_FLAG_REFINE: F += forward(f - inverse(F)), inverse and difference in FP64):
    # inverse + refined forward of a few functions of the batch, pairs/s per function
    refined = None
    if not args.no_accuracy:
        rb = min(b, 8)
        pr = _lib.Plan(_lib.SO3_COMPLEX, L, rb, "tc_bf16x3", "stable", _lib.FLAG_REFINE)
        gr = torch.empty(rb * N ** 3, dtype=torch.complex64, device=dev)
        cr = torch.empty(rb * C, dtype=torch.complex64, device=dev)
        pr.inverse(coef[:rb * C].data_ptr(), gr.data_ptr(), sp)
        pr.forward(grid[:rb * N ** 3].data_ptr(), cr.data_ptr(), sp)
        torch.cuda.synchronize()
        pr.set_timing(True)
        pr.stage_times(reset=True)
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r0.record(stream)
        pr.inverse(coef[:rb * C].data_ptr(), gr.data_ptr(), sp)
        pr.forward(grid[:rb * N ** 3].data_ptr(), cr.data_ptr(), sp)
        r1.record(stream)
        torch.cuda.synchronize()
        pr.check()
        rst = pr.stage_times(reset=True)
        rms_ = r0.elapsed_time(r1)
        refined = {"value": rb * 1000.0 / rms_, "unit": UNIT, "batch": rb, "ms_per_step": rms_,
                   "forward_rel_rms": acc.get("refined_forward_rel_rms"),
                   "forward_rel_max_per_l": acc.get("refined_forward_rel_max_per_l"),
                   "stages_ms": {k: v for k, (v, _) in rst.items()},
                   "note": "tensor-core inverse + refined forward (FFTSO3_FLAG_REFINE: the inverse of the first "
                           "result exactly on the tensor cores (BF16 digit products summed without rounding) and "
                           "f - inverse(F) in double-float, then the tensor-core forward of the residual)"}
        del pr, gr, cr
        torch.cuda.empty_cache()

    cpu = None
    if not args.no_cpu:
        cpu = cpu_baselines(L)

    if rank == 0:
        metric = METRIC if L == 255 else METRIC.replace("l_max=255", f"l_max={L}")
        line = {
            "metric": metric, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16x3 (split) / fp32 accumulate / fp32 FFT", "data": "synthetic",
            "config": {"workload": f"SO(3) complex forward+inverse, l_max={L}, batch={b} functions per GPU "
                                   f"({N}^3 complex64 grid each), TC split-BF16, stable recursion",
                       "l_max": L, "batch_per_gpu": b, "precision": "tc_bf16x3",
                       "l2": "inputs larger than L2 (1 GB grid per function)"},
            "e2e": e2e, "gpu_launches": launches, "roofline": roof, "step_roofline": step_roof,
            "stages": stage_summary,
            "accuracy": acc, "refined_path": refined, "fp64_path": fp64, "fp32_cuda_core_path": fp32,
            "speedup_vs_fp64_path": value / fp64["value"] if fp64 else None,
            "clocks": clocks, "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
