#!/usr/bin/env python
"""Benchmark: SO(3) forward+inverse transform pairs per second at l_max = 255.

Headline (the first JSON line): a batch of 32 complex SO(3) functions at
l_max = 255 (512^3 Euler grid each, complex64 samples; synthetic seeded
coefficients F ~ N(0,1)(l+1)^-1.5), stable Wigner-d recursion.  One step =
inverse of the whole batch on the tensor cores (split-BF16) + refined forward
of the whole batch (F0 = split-BF16 GEMM of the samples' double-float FFT,
then one residual step F = F0 + GEMM(FFT(f) - N^2 H(F0)) formed in the pencil
domain, H the exact tensor-core synthesis contraction), the configuration that
meets rel-err <= 1e-6 per degree against FP64; value = functions / step time.  Reported beside it: the plain split-BF16 step, the
plain FP64 GPU path, the FP32 CUDA-core form, the accuracy against FP64, the
end-to-end rate through the host-buffer C-ABI calls, the roofline of the
dominant stage (CUDA-event stage timing inside the library) and of the whole
step, and the CPU baseline: the oracle's restatement of the reference
algorithm on beta slices spread over [0, pi), at all host threads and at one.

Then (--workload all, the default) one line per other configuration: the
plain FP64 path at l_max = 127, 4096 real functions of uneven bandwidth, 256
complex functions at l_max = 96, and 512 real S^2 signals at l_max = 511,
each with its accuracy, roofline and CPU baseline.

The library runs on one GPU (no sharding, no collectives): launched with more
than one rank, rank 0 prints a line saying so and no GPU work is done.
--impl reference times only the CPU algorithm (all host threads) on the
headline workload and prints its own JSON line.
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
    this workload: by batch (functions per launch) at the same l_max, and for
    the FFT stages (whose traffic is one read and one write of every sample) by
    batch * N^3 across l_max."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    found = [(r["l_max"], r["batch"], r["bytes_per_launch"]) for r in json.load(open(path))["captures"]
             if r["stage"] == stage]
    for L0, b0, byts in found:
        if L0 == l_max:
            return byts * batch / b0
    for L0, b0, byts in found:
        if "fft" in stage:
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


def uneven_line(args) -> dict:
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
    acc_rms, acc_max, acc_idx = [], [], []
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
        acc_max.append(per_l_errors(a.cpu().numpy(), ci.cpu().numpy(), L)[1])
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
    # roofline of the dominant stage of the eager step: FFT stages against HBM (one complex64 read + write of the
    # work grid per pass, both directions, summed over the buckets that use the stage), GEMMs against BF16
    top, (top_ms, _) = max(st_all.items(), key=lambda kv: kv[1][0])
    bsz = {}
    for k in range(bt.buckets):
        Lb, cnt = bt.bucket_info(k)
        bsz[Lb] = cnt
    if top == "fft_slices":
        # both passes of every beta slice in one launch per direction: the real grid read (or written) once and
        # the complex64 pencils written (or read) once, 4 + 8 B per sample and direction
        byts = sum(2 * 12.0 * (2 * (Lb + 1)) ** 3 * c for Lb, c in bsz.items())
        ach = byts / (top_ms / 1000.0) / 1e9
        roof = {"bound": "hbm", "unit": "GB/s", "achieved": ach, "peak": peaks["hbm_gbs"],
                "frac": ach / peaks["hbm_gbs"],
                "algorithmic": "real FP32 grid + complex64 pencils, once each per direction (12 B per sample)"}
    elif top == "coeff_convert":
        byts = sum(2 * 12.0 * ((Lb + 1) * (4 * (Lb + 1) ** 2 - 1) // 3) * c for Lb, c in bsz.items())
        ach = byts / (top_ms / 1000.0) / 1e9
        roof = {"bound": "hbm", "unit": "GB/s", "achieved": ach, "peak": peaks["hbm_gbs"],
                "frac": ach / peaks["hbm_gbs"],
                "algorithmic": "complex64 group-major + real FP32 packed coefficients, once each per direction"}
    elif top.startswith("tc_gemm"):
        fl = sum(8.0 * (Lb + 1) * ((Lb + 1) * (4 * (Lb + 1) ** 2 - 1) // 3) * c for Lb, c in bsz.items()
                 if top in dict((L2, d) for _, L2, _, d in per_bucket).get(Lb, {}))
        ach = fl / (top_ms / 1000.0) / 1e12
        roof = {"bound": "tensor", "unit": "TFLOP/s", "achieved": ach, "peak": peaks["bf16_tflops_sustained"],
                "frac": ach / peaks["bf16_tflops_sustained"], "algorithmic": "8 B C useful flops per function"}
    else:
        byts = sum(2 * 16.0 * (2 * (Lb + 1)) ** 3 * c for Lb, c in bsz.items()
                   if top in dict((L2, d) for _, L2, _, d in per_bucket).get(Lb, {}))
        ach = byts / (top_ms / 1000.0) / 1e9
        roof = {"bound": "hbm", "unit": "GB/s", "achieved": ach, "peak": peaks["hbm_gbs"],
                "frac": ach / peaks["hbm_gbs"],
                "algorithmic": "one complex64 read + write of each bucket's work grid per pass, both directions"}
    roof.update({"kernel": top, "ms_per_step": top_ms, "peak_source": peaks["source"], "traffic": None,
                 "share_of_eager_step": top_ms / sum(v for v, _ in st_all.values())})
    # CPU baseline: the oracle (the reference algorithm restated) on functions spread over the batch
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O

        O.build()
        nth = os.cpu_count() or 1
        O.set_num_threads(nth)
        idx = np.linspace(0, n - 1, 8).astype(int)
        t_sum = 0.0
        for i in idx:
            Li = int(lmax[i])
            Fi = coef[bt.coeff_offset(i):bt.coeff_offset(i) + (Li + 1) * (4 * (Li + 1) ** 2 - 1) // 3].double().cpu().numpy()
            t0 = time.perf_counter()
            gi = O.so3_inverse_real_grid(Li, Fi)
            O.so3_forward_real(Li, gi)
            t_sum += time.perf_counter() - t0
        cpu = {"value": len(idx) / t_sum, "unit": UNIT, "cores": nth, "kind": "port",
               "sample": f"{len(idx)} functions spread over the batch (l_max {sorted(int(lmax[i]) for i in idx)}), "
                         f"real inverse on the grid + real forward each (oracle restatement of "
                         f"fdcl_FFTSO3.cpp:774-850 / :1141-1167, OpenMP over beta slices, {nth} threads); pairs/s "
                         f"per function"}
    line = {
        "metric": UNEVEN_METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16x3 (split) / fp32 accumulate / fp32 FFT; fp32 samples",
        "data": "synthetic",
        "config": {"workload": f"{n} real SO(3) functions, l_max uniform in 8..64 (seed 3), coefficients "
                               "N(0,1)/(2l+1), FP32 samples; fftso3_batch, tensor-core buckets, CUDA graph",
                   "functions": n, "buckets": bt.buckets, "streams": bt.streams, "samples": int(G),
                   "coefficients": int(Ctot),
                   "form": ("three launches per direction over all buckets (slice FFT, fused GEMM, conversion)"
                            if bt.graph_kernels(0) == 3 else "per-bucket phases around one fused GEMM launch"),
                   "l2": "inputs larger than L2"},
        "io_gbs": io_bytes / (ms / 1000.0) / 1e9, "io_frac_of_hbm": io_bytes / (ms / 1000.0) / 1e9 / peaks["hbm_gbs"],
        "batch_create_s": t_create, "device_gb": bt.device_bytes / 1e9,
        "accuracy": {"rel_rms_vs_fp64_max": max(acc_rms), "rel_max_per_l_vs_fp64_max": max(acc_max),
                     "functions": acc_idx, "against": "FP64 GPU plans (FFTSO3_REAL) on the same FP32 samples"},
        "roofline": roof, "cpu_baseline": cpu,
        "fp64_loop": fp64, "speedup_vs_fp64_loop": value / fp64["value"] if fp64 else None,
        "clocks": clocks, "gpu_launches": launches * args.steps,
        "stages_eager_sum_ms": stage_summary, "eager_timed_step_ms": eager_ms,
        "graph_kernels": {"forward": bt.graph_kernels(0), "inverse": bt.graph_kernels(1)},
    }
    if per_bucket and per_bucket[0][0] > 0:  # the per-bucket form: the costliest buckets
        line["top_buckets"] = [{"l_max": L, "functions": c, "ms": t, "stages": d} for t, L, c, d in per_bucket[:6]]
    return line


# --------------------------------------------------------------- FP64 plain path

FP64_METRIC = "SO(3) FP64 fwd+inv transforms/s at l_max={L}: plain FP64 GPU path (complex and real)"


def fp64_line(args) -> dict:
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
    # roofline of the complex step's dominant stage: an FFT pass against HBM, or the contraction against FP64
    peaks = measured_peaks()
    cx = out["complex"]
    top = max(cx["stages_ms"].items(), key=lambda kv: kv[1])[0]
    if top in cx["fft"]:
        gbs = cx["fft"][top]["gbs"]
        roof = {"bound": "hbm", "unit": "GB/s", "kernel": f"fft_lines_kernel (FP64, {top})", "achieved": gbs,
                "peak": peaks["hbm_gbs"], "frac": gbs / peaks["hbm_gbs"], "peak_source": peaks["source"],
                "ms_per_launch": cx["fft"][top]["ms_per_launch"], "traffic": None,
                "algorithmic": "one complex128 read + write of the grid per pass"}
    else:
        tf = cx["contraction"][top]["fp64_tflops"]
        roof = {"bound": "fp64", "unit": "TFLOP/s", "kernel": top, "achieved": tf, "peak": FP64_NOMINAL_TFLOPS,
                "frac": tf / FP64_NOMINAL_TFLOPS, "peak_source": "nominal FP64 (no measured FP64 peak)",
                "ms_per_launch": cx["contraction"][top]["ms_per_launch"], "traffic": None,
                "algorithmic": "8 B C flops per direction"}
    # parity with the reference's algorithm: the oracle (CPU restatement) on one complex function
    parity = None
    if not args.no_accuracy:
        from oracle import oracle as O

        O.build()
        O.set_num_threads(os.cpu_count() or 1)
        rng = np.random.Generator(np.random.PCG64(7))
        l = np.concatenate([np.full((2 * x + 1) ** 2, x) for x in range(B)])
        F = (rng.standard_normal(C) + 1j * rng.standard_normal(C)) / (2 * l + 1)
        g_or = O.so3_inverse_complex_grid(L, F)
        F_or = O.so3_forward_complex(L, g_or)
        p = _lib.Plan(_lib.SO3_COMPLEX, L, 1, "fp64", "reference")
        c = torch.from_numpy(F).to(dev)
        g = torch.empty(N ** 3, dtype=torch.complex128, device=dev)
        p.inverse(c.data_ptr(), g.data_ptr(), sp)
        gin = torch.from_numpy(np.ascontiguousarray(g_or).ravel()).to(dev)
        c2 = torch.empty_like(c)
        p.forward(gin.data_ptr(), c2.data_ptr(), sp)
        torch.cuda.synchronize()
        p.check()
        gg = g.cpu().numpy().reshape(N, N, N)
        rf, mf = per_l_errors(c2.cpu().numpy(), F_or, L)
        parity = {"inverse_rel_rms": float(np.linalg.norm(gg - g_or) / np.linalg.norm(g_or)),
                  "forward_rel_rms": rf, "forward_rel_max_per_l": mf,
                  "against": "the oracle (reference algorithm restated in C, FP64, reference recursion) on one "
                             "complex function, coefficients N(0,1)/(2l+1)"}
        del p, c, g, gin, c2
    cpu = cpu_baselines(L) if not args.no_cpu else None
    line = {"metric": FP64_METRIC.format(L=L), "value": out["complex"]["pairs_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["complex"]["ms_per_pair"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"one SO(3) function, l_max={L} ({N}^3 grid), FP64, reference recursion; "
                                   "coefficients N(0,1)/(2l+1)"},
            "roofline": roof, "accuracy": parity, "cpu_baseline": cpu,
            "complex": out["complex"], "real": out["real"]}
    return line


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


def s2_line(args) -> dict:
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
    # roofline of the dominant stage of one eager step
    top, (top_ms, top_n) = max(stages.items(), key=lambda kv: kv[1][0])
    if top in gemm:
        roof = {"bound": "tensor", "unit": "TFLOP/s", "achieved": gemm[top]["tflops"],
                "peak": peaks["bf16_tflops_sustained"], "frac": gemm[top]["frac_of_bf16"],
                "algorithmic": "4 N B^2 useful flops per signal"}
    elif top in fft:
        roof = {"bound": "hbm", "unit": "GB/s", "achieved": fft[top]["gbs"], "peak": peaks["hbm_gbs"],
                "frac": fft[top]["frac_of_hbm"], "algorithmic": "real samples (4 B) + complex pencils (8 B) per pass"}
    else:
        roof = {"bound": "hbm", "unit": "GB/s", "achieved": None, "peak": peaks["hbm_gbs"], "frac": None}
    roof.update({"kernel": top, "ms_per_launch": top_ms / top_n, "peak_source": peaks["source"], "traffic": None,
                 "share_of_eager_step": top_ms / sum(v for v, _ in stages.values())})
    # per-degree error of the forward (rel_max = max_l max_m |a - b| / rms_m |b|)
    a0 = coef_out[0].double().cpu().numpy()
    b0 = F64.cpu().numpy()
    mx = 0.0
    for ll in range(B):
        sl = slice(ll * ll, (ll + 1) * (ll + 1))
        mx = max(mx, float(np.abs(a0[sl] - b0[sl]).max() / np.sqrt(np.mean(b0[sl] ** 2))))
    acc["forward_rel_max_per_l"] = mx
    # CPU baseline: the oracle on one signal (real inverse on the grid + real forward)
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O

        O.build()
        nth = os.cpu_count() or 1
        O.set_num_threads(nth)
        Fs = coef[0].double().cpu().numpy()
        t0 = time.perf_counter()
        gs = O.s2_inverse_real_grid(L, Fs)
        O.s2_forward_real(L, gs)
        dt = time.perf_counter() - t0
        cpu = {"value": 1.0 / dt, "unit": UNIT, "cores": nth, "kind": "port",
               "sample": f"one signal at l_max={L}: real inverse on the grid + real forward (oracle restatement of "
                         f"fdcl_FFTS2.cpp:424-436 / :500-512, OpenMP over theta, {nth} threads)"}
    line = {
        "metric": S2_METRIC.format(b=b, L=L), "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16x3 (split) / fp32 accumulate / fp32 FFT; fp32 samples", "data": "synthetic",
        "config": {"workload": f"{b} real S^2 signals, l_max={L} ({N}x{N} grid, FP32 samples), coefficients "
                               "N(0,1)/(l+1); FFTS2_real tensor-core plan", "signals": b, "l_max": L,
                   "l2": "inputs larger than L2 (2 GB of samples)"},
        "accuracy": acc, "fp64_path": fp64, "speedup_vs_fp64_path": value / fp64["value"],
        "roofline": roof, "cpu_baseline": cpu, "gemm": gemm, "fft": fft,
        "stages": {k: {"ms": v, "launches": c} for k, (v, c) in stages.items()},
        "gpu_launches": int(sum(c for _, c in stages.values())) * args.steps, "clocks": clocks,
    }
    return line


# --------------------------------------------------------------- GPU arm

def stage_roofline(name: str, tot_ms: float, cnt: int, L: int, b: int, chunk: int, peaks: dict, piece: int = 0):
    """Achieved rate of one stage of an SO(3) complex tensor-core plan from its CUDA-event time, against the
    measured peak: algorithmic bytes (HBM-bound stages) or useful flops (contractions) per timed record."""
    B, N = L + 1, 2 * (L + 1)
    C = B * (4 * B * B - 1) // 3
    per = tot_ms / cnt / 1000.0
    grid8 = 8.0 * b * N ** 3
    flops = None
    if name.startswith("tc_gemm"):
        flops, alg = 8.0 * B * C * b, "8 B C useful flops per function per launch (6 split-BF16 products issued)"
    elif name in ("refine_exact_contract", "exact_inverse_contract"):
        flops, alg = 8.0 * B * C * chunk, "8 B C useful flops per function of the chunk (10 digit products issued)"
    if flops is not None:
        ach = flops / per / 1e12
        return {"bound": "tensor", "unit": "TFLOP/s", "kernel": name, "achieved": ach,
                "peak": peaks["bf16_tflops_sustained"], "frac": ach / peaks["bf16_tflops_sustained"],
                "peak_source": peaks["source"] + " (sustained bf16)", "ms_per_launch": per * 1000.0,
                "algorithmic": alg}
    if name == "fft_2d":
        byts, alg = 2 * grid8, "one complex64 read + write of every sample per launch (both FFT passes, L2 ring)"
    elif name in ("fft_rows", "fft_cols", "tc_pack_fwd", "tc_pack_inv"):
        byts, alg = 2 * grid8, "one complex64 read + write of every sample per pass"
    elif name == "refine_fft_df32":
        byts, alg = (8.0 + 16 + 16 + 16) * (piece or chunk) * N ** 3, ("double-float forward FFT of the samples: pass 1 reads "
                                                          "8 B, writes 16 B; pass 2 reads 16 B, writes hi + lo "
                                                          "8 + 8 B per sample")
    elif name == "exact_inverse_fft_df32":
        byts, alg = (16.0 + 16 + 16 + 8) * (piece or chunk) * N ** 3, ("double-float FFT of the synthesis: pass 1 "
                                                                    "reads and writes 16 B; pass 2 reads 16 B, "
                                                                    "writes the complex64 grid (8 B) per sample")
    elif name == "basis_convert":
        byts, alg = 2 * 8.0 * C * b, "one complex64 read + write of the coefficients"
    else:
        byts, alg = None, "mixed elementwise work"
    ach = byts / per / 1e9 if byts else None
    return {"bound": "hbm", "unit": "GB/s", "kernel": name, "achieved": ach, "peak": peaks["hbm_gbs"],
            "frac": ach / peaks["hbm_gbs"] if ach else None, "peak_source": peaks["source"],
            "ms_per_launch": per * 1000.0, "algorithmic": alg}


def so3_tc_line(args, L: int, b: int, full: bool = True) -> dict:
    """One SO(3) complex batch on the tensor cores: b functions at l_max = L, one step = inverse + forward of
    the batch.  full (the headline): the forward carries the residual refinement (FFTSO3_FLAG_REFINE), so the
    step meets rel-err <= 1e-6 under the per-degree metric; the end-to-end host-buffer rate, the plain
    split-BF16 step and the FP32 CUDA-core form are reported beside it.  Otherwise (full = False) the plain
    split-BF16 step with its accuracy against FP64, the FP64 path, roofline and CPU baseline."""
    import torch

    import fftso3_gb300 as fg
    from fftso3_gb300 import _lib
    from fftso3_gb300 import build as fbuild

    fbuild.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    N = 2 * (L + 1)
    B = L + 1
    C = fg.so3_ncoeff(L)
    peaks = measured_peaks()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # ---- FP64 plain path: reference data for the accuracy checks (function 0) and its own rate
    F0 = seeded_coeffs(L, 0)
    fp64 = None
    have_ref = not args.no_accuracy
    g0_c64 = F0_fp64 = g0_ref = None
    if have_ref:
        p64 = _lib.Plan(_lib.SO3_COMPLEX, L, 1, "fp64", "stable")
        c64 = torch.from_numpy(F0).to(dev)
        g64 = torch.empty(N ** 3, dtype=torch.complex128, device=dev)
        o64 = torch.empty_like(c64)
        p64.inverse(c64.data_ptr(), g64.data_ptr(), sp)
        p64.forward(g64.data_ptr(), o64.data_ptr(), sp)
        torch.cuda.synchronize()
        F0_fp64 = o64.cpu().numpy()  # FP64 forward of the FP64 synthesis
        g0_c64 = g64.to(torch.complex64)
        g0_ref = g64.cpu().numpy()
        if not args.no_fp64:
            reps = 2
            e0, e1 = ev(), ev()
            e0.record(stream)
            for _ in range(reps):
                p64.inverse(c64.data_ptr(), g64.data_ptr(), sp)
                p64.forward(g64.data_ptr(), o64.data_ptr(), sp)
            e1.record(stream)
            torch.cuda.synchronize()
            ms64 = e0.elapsed_time(e1) / reps
            fp64 = {"value": 1000.0 / ms64, "unit": UNIT, "ms_per_pair": ms64, "batch": 1,
                    "note": "plain FP64 GPU path (FFTSO3_PREC_FP64, stable recursion), same l_max"}
        del p64, g64, o64, c64
        torch.cuda.empty_cache()

    # ---- inputs: b seeded band-limited functions (function 0: the FP64 synthesis, rounded to complex64)
    Fb = np.concatenate([seeded_coeffs(L, i) for i in range(b)]).astype(np.complex64)
    coef = torch.from_numpy(Fb).to(dev)
    grid = torch.empty(b * N ** 3, dtype=torch.complex64, device=dev)
    coef_out = torch.empty_like(coef)
    grid_out = torch.empty_like(grid)

    def accuracy(plan):
        """forward of function 0's complex64 grid and inverse of its coefficients, against FP64"""
        coef_in = coef.clone()
        coef_in[:C].copy_(torch.from_numpy(F0.astype(np.complex64)).to(dev))
        plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
        plan.inverse(coef_in.data_ptr(), grid_out.data_ptr(), sp)
        torch.cuda.synchronize()
        plan.check()
        fr, fm = per_l_errors(coef_out[:C].cpu().numpy().astype(np.complex128), F0_fp64, L)
        gi = grid_out[:N ** 3].cpu().numpy().astype(np.complex128)
        ir = float(np.linalg.norm(gi - g0_ref) / np.linalg.norm(g0_ref))
        im = float(np.abs(gi - g0_ref).max() / np.sqrt(np.mean(np.abs(g0_ref) ** 2)))
        del coef_in
        return {"forward_rel_rms": fr, "forward_rel_max_per_l": fm, "inverse_rel_rms": ir, "inverse_rel_max": im}

    def timed(plan, steps, warmup, clocks=False):
        for _ in range(warmup):
            plan.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
            plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
        torch.cuda.synchronize()
        plan.set_timing(True)
        plan.stage_times(reset=True)
        e0, e1 = ev(), ev()
        clk = ClockSampler(0) if clocks else None
        if clk:
            clk.__enter__()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            plan.inverse(coef.data_ptr(), grid_out.data_ptr(), sp)
            plan.forward(grid.data_ptr(), coef_out.data_ptr(), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        if clk:
            clk.__exit__(None, None, None)
        t = e0.elapsed_time(e1) / steps
        st = plan.stage_times(reset=True)
        plan.set_timing(False)
        plan.check()
        return t, st, (clk.summary() if clk else None)

    # ---- the measured plan: refined forward and exact inverse (headline) or plain split-BF16
    flags = _lib.FLAG_AUTOTUNE | (_lib.FLAG_REFINE | _lib.FLAG_EXACT_INVERSE if full else 0)
    plan = _lib.Plan(_lib.SO3_COMPLEX, L, b, "tc_bf16x3", "stable", flags)
    plan.inverse(coef.data_ptr(), grid.data_ptr(), sp)  # synthetic band-limited FP32 samples
    if have_ref:
        grid[:N ** 3].copy_(g0_c64)
    torch.cuda.synchronize()
    plan.check()
    acc = accuracy(plan) if have_ref else {}
    if have_ref:
        acc["against"] = "FP64 GPU path (stable recursion) on the same function (function 0 of the batch)"
        if full:  # the names of the refined forward's figures
            acc["refined_forward_rel_rms"] = acc["forward_rel_rms"]
            acc["refined_forward_rel_max_per_l"] = acc["forward_rel_max_per_l"]
    ms, stages, clocks = timed(plan, args.steps, args.warmup, clocks=True)
    value = b * 1000.0 / ms
    # functions per refinement chunk (the library sizes chunks to the free device memory): one timed record of
    # the refinement FFT per chunk and step
    nchunks = max(1, round(stages.get("refine_exact_contract", (0, args.steps))[1] / args.steps))
    chunk = -(-b // nchunks)  # functions per exact-contraction launch
    npieces = max(1, round(stages.get("refine_fft_df32", (0, args.steps))[1] / args.steps))
    piece = -(-b // npieces)  # functions per double-float FFT record
    nichunks = max(1, round(stages.get("exact_inverse_contract", (0, args.steps))[1] / args.steps))
    ichunk = -(-b // nichunks)  # functions per exact-inverse chunk (contraction and double-float FFT records)
    nrec = int(sum(c for _, c in stages.values()))
    # kernels in the timed region: one per timed record, plus the second kernel of the records that hold two
    # (the double-float FFTs' two passes; the gather and Nyquist zeroing before each exact-inverse contraction)
    # (each contraction's gather record also holds its digit-image kernel, the exact inverse's its Nyquist zeroing)
    launches = nrec + int(stages.get("refine_fft_df32", (0, 0))[1]) + \
        int(stages.get("exact_inverse_fft_df32", (0, 0))[1]) + 2 * int(stages.get("exact_inverse_contract", (0, 0))[1]) + \
        int(stages.get("refine_exact_contract", (0, 0))[1])
    tot = sum(v for v, _ in stages.values())
    stage_summary = {k: {"ms_per_launch": v / c, "launches": c, "share": v / tot} for k, (v, c) in stages.items()}
    top, (top_ms, top_n) = max(stages.items(), key=lambda kv: kv[1][0])
    per_record = {"refine_fft_df32": piece, "refine_exact_contract": chunk, "exact_inverse_fft_df32": ichunk,
                  "exact_inverse_contract": ichunk}
    roof = stage_roofline(top, top_ms, top_n, L, b, per_record.get(top, chunk), peaks, per_record.get(top, 0))
    roof["traffic"] = profiled_traffic(top, L, per_record.get(top, b))  # functions per launch record
    roof["share_of_step"] = top_ms / tot

    # ---- the step against its floors: HBM (algorithmic bytes of every stage) and tensor (issued MMA flops)
    Kp = (N + 63) // 64 * 64
    table_rows = sum((2 * m + 1) * (B - m) for m in range(B))
    table_b = 3 * 2.0 * Kp * table_rows        # three BF16 planes, read once per split-BF16 GEMM launch
    coef_b = 8.0 * b * C
    grid_b = 8.0 * b * N ** 3
    useful = 8.0 * B * C * b
    gemm_dir = (grid_b + table_b + coef_b) + 2 * coef_b  # GEMM + permutation, one direction
    tc_dir = 2 * grid_b + gemm_dir                         # with the FFT
    step_bytes = 2 * tc_dir
    tensor_flops = 2 * 6 * useful
    if full:
        # the refined forward replaces the split-BF16 forward: double-float FFT of the samples, GEMM of its FP32
        # part, exact synthesis contraction with the pencil-domain residual, GEMM of the residual, correction
        oz_table = nchunks * 4 * 2.0 * Kp * table_rows   # digit planes, read once per chunk launch
        step_bytes += (-tc_dir
                       + 7 * grid_b                                # FFT: 8 B in, 16 + 16 B, hi + lo out
                       + gemm_dir                                  # F0
                       + coef_b + 2 * 16.0 * b * C                 # gather: coefficients in, double-float runs out
                       + oz_table + 16.0 * b * C + 3 * grid_b      # contraction: table, runs, hi + lo in, r out
                       + gemm_dir                                  # the residual's forward
                       + 3 * coef_b)                               # correction added
        tensor_flops += 6 * useful + 10 * useful
        # the exact inverse replaces the split-BF16 inverse: gather, exact synthesis contraction (digit planes per
        # chunk, double-float runs in, double-float pencils out), double-float FFT rounded into the grid
        step_bytes += (-tc_dir
                       + coef_b + 2 * 16.0 * b * C                 # gather
                       + nichunks * 4 * 2.0 * Kp * table_rows      # digit planes
                       + 16.0 * b * C + 2 * grid_b                 # runs in, 16 B per pencil place out
                       + 7 * grid_b)                               # FFT: 16 + 16 B, then 16 B in, 8 B out
        tensor_flops += -6 * useful + 10 * useful
    hbm_floor_ms = step_bytes / (peaks["hbm_gbs"] * 1e9) * 1e3
    tensor_floor_ms = tensor_flops / (peaks["bf16_tflops_sustained"] * 1e12) * 1e3
    floor_ms = max(hbm_floor_ms, tensor_floor_ms)
    step_roof = {"bound": "hbm" if hbm_floor_ms >= tensor_floor_ms else "tensor", "algorithmic_bytes": step_bytes,
                 "hbm_floor_ms": hbm_floor_ms, "tensor_floor_ms": tensor_floor_ms, "ms_per_step": ms,
                 "frac": floor_ms / ms, "peak_source": peaks["source"],
                 "note": "split-BF16 directions: FFT 2 x grid bytes, GEMM pencils + BF16 table + coefficients, "
                         "permutation 2 x coefficients" + ("; refined forward: double-float FFT of the samples "
                                                           "(56 B per sample), two GEMMs + permutations, the "
                                                           "exact synthesis contraction (digit planes per chunk, "
                                                           "double-float runs, 24 B per sample of pencils) and "
                                                           "the correction; exact inverse: the exact synthesis "
                                                           "contraction (16 B per pencil place out) and the "
                                                           "double-float FFT (56 B per sample)" if full else "")}

    # ---- end to end through the host-buffer C ABI (pinned host memory), the same plan and step count
    e2e = None
    if full and not args.no_e2e:
        hg = torch.empty(b * N ** 3, dtype=torch.complex64, pin_memory=True)
        hg.copy_(grid)
        hc = torch.empty(b * C, dtype=torch.complex64, pin_memory=True)
        hc.copy_(coef)
        hco = torch.empty_like(hc, pin_memory=True)
        # the inverse writes the grid the forward then reads (one pinned grid buffer)
        plan.inverse_host(hc.data_ptr(), hg.data_ptr(), sp)
        plan.forward_host(hg.data_ptr(), hco.data_ptr(), sp)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            plan.inverse_host(hc.data_ptr(), hg.data_ptr(), sp)
            plan.forward_host(hg.data_ptr(), hco.data_ptr(), sp)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / args.steps
        e2e = {"value": b / dt, "unit": UNIT, "h2d_bytes_per_step": int(8 * b * C + 8 * b * N ** 3),
               "d2h_bytes_per_step": int(8 * b * N ** 3 + 8 * b * C), "steps": args.steps}
        del hg, hc, hco
    plan.close()
    del plan
    torch.cuda.empty_cache()

    # ---- beside the headline: the refined forward with the split-BF16 inverse, the plain split-BF16 step (no
    # refinement) and the FP32 CUDA-core form
    plain = fp32 = fwdonly = None
    if full:
        pf = _lib.Plan(_lib.SO3_COMPLEX, L, b, "tc_bf16x3", "stable", _lib.FLAG_AUTOTUNE | _lib.FLAG_REFINE)
        facc = accuracy(pf) if have_ref else {}
        fms, fst, _ = timed(pf, args.steps, min(args.warmup, 3))
        fwdonly = {"value": b * 1000.0 / fms, "unit": UNIT, "ms_per_step": fms, "accuracy": facc,
                   "stages": {k: {"ms_per_launch": v / c, "launches": c} for k, (v, c) in fst.items()},
                   "note": "FFTSO3_FLAG_REFINE only: the refined forward meets 1e-6 per degree, the split-BF16 "
                           "inverse's FP32 FFT leaves grid errors above 1e-6 of the rms (inverse_rel_max)"}
        pf.close()
        del pf
        torch.cuda.empty_cache()
        pp = _lib.Plan(_lib.SO3_COMPLEX, L, b, "tc_bf16x3", "stable", _lib.FLAG_AUTOTUNE)
        pacc = accuracy(pp) if have_ref else {}
        pms, pst, _ = timed(pp, args.steps, min(args.warmup, 3))
        ptop, (ptop_ms, ptop_n) = max(pst.items(), key=lambda kv: kv[1][0])
        proof = stage_roofline(ptop, ptop_ms, ptop_n, L, b, chunk, peaks)
        proof["traffic"] = profiled_traffic(ptop, L, b)
        plain = {"value": b * 1000.0 / pms, "unit": UNIT, "ms_per_step": pms, "accuracy": pacc, "roofline": proof,
                 "stages": {k: {"ms_per_launch": v / c, "launches": c} for k, (v, c) in pst.items()},
                 "note": "split-BF16 forward and inverse without the residual step: its forward meets 1e-6 as "
                         "rel_rms but not per degree (rel_max)"}
        pp.close()
        del pp
        torch.cuda.empty_cache()
        if not args.no_fp32:
            p32 = _lib.Plan(_lib.SO3_COMPLEX, L, b, "fp32", "stable")
            a32 = accuracy(p32) if have_ref else {}
            ms32, _, _ = timed(p32, 1, 1)
            fp32 = {"value": b * 1000.0 / ms32, "unit": UNIT, "ms_per_step": ms32, "accuracy": a32,
                    "note": "FFTSO3_PREC_FP32: FP32 table and FMA accumulation on the CUDA cores, same batch"}
            p32.close()
            del p32
            torch.cuda.empty_cache()

    cpu = cpu_baselines(L) if not args.no_cpu else None
    metric = METRIC if L == 255 else METRIC.replace("l_max=255", f"l_max={L}")
    what = ("exact inverse (exact tensor-core synthesis contraction, double-float FFT, one rounding to complex64) + "
            "refined forward (double-float FFT of the samples, split-BF16 GEMM, the residual against the exact "
            "tensor-core synthesis formed in the pencil domain, split-BF16 GEMM of the residual)"
            if full else "inverse + forward, split-BF16")
    line = {
        "metric": metric, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16x3 (split) / fp32 accumulate / fp32 FFT" +
                                      ("; refined forward and exact inverse: double-float FFTs, exact BF16 digit "
                                       "products" if full else ""),
        "data": "synthetic",
        "config": {"workload": f"SO(3) complex, l_max={L}, batch={b} functions ({N}^3 complex64 grid each), stable "
                               f"recursion; one step = {what}",
                   "l_max": L, "batch": b, "precision": "tc_bf16x3" + (" + refine + exact inverse" if full else ""),
                   "refine_chunk": chunk if full else None, "refine_fft_piece": piece if full else None,
                   "exact_inverse_chunk": ichunk if full else None,
                   "l2": f"inputs larger than L2 ({8.0 * b * N ** 3 / 1e9:.1f} GB of complex64 grids)"},
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "step_roofline": step_roof,
        "stages": stage_summary, "accuracy": acc, "fp64_path": fp64,
        "speedup_vs_fp64_path": value / fp64["value"] if fp64 else None,
        "clocks": clocks, "cpu_baseline": cpu,
    }
    if full:
        line["refined_forward_plain_inverse_path"] = fwdonly
        line["unrefined_path"] = plain
        line["fp32_cuda_core_path"] = fp32
    return line


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
    ap.add_argument("--workload", default="all",
                    choices=["all", "lmax255", "uneven", "s2", "fp64", "lmax96", "fft", "points"],
                    help="all (default): the headline line (SO(3) l_max=255 batch) first, then one line per other "
                         "configuration (fp64, uneven, lmax96, s2); lmax255: the headline SO(3) batch at one l_max "
                         "(--l-max/--batch) alone; uneven: the mixed-bandwidth SO(3) batch; s2: the S^2 batch at "
                         "l_max=511; fp64: the plain FP64 path at l_max=127; lmax96: 256 complex SO(3) functions at "
                         "l_max=96")
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
    if args.workload == "fft":
        main_fft(args)
        return
    if args.workload == "points":
        main_points(args)
        return
    run_workload(args)


CONFIG_LINES = {
    "fp64": lambda a: fp64_line(a),
    "uneven": lambda a: uneven_line(a),
    "lmax96": lambda a: so3_tc_line(a, 96, 256, full=False),
    "s2": lambda a: s2_line(a),
}


def run_workload(args) -> None:
    """The headline line first (the one the driver parses); with --workload all, then one line per other
    configuration, each freeing its GPU memory before the next (a failure there prints an error line)."""
    import gc

    if args.workload not in ("all", "lmax255"):
        print(json.dumps(CONFIG_LINES[args.workload](args)), flush=True)
        return
    print(json.dumps(so3_tc_line(args, args.l_max, args.batch, full=True)), flush=True)
    if args.workload != "all":
        return
    import torch

    for name, fn in CONFIG_LINES.items():
        gc.collect()
        torch.cuda.empty_cache()
        try:
            print(json.dumps(fn(args)), flush=True)
        except Exception as e:  # report and go on: the headline is already out
            print(json.dumps({"workload": name, "error": f"{type(e).__name__}: {e}"}), flush=True)


if __name__ == "__main__":
    main()
