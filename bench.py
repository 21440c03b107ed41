#!/usr/bin/env python
"""Benchmark of the GB300 dense LU solve path.

Headline metric: n=32768 DGESV time-to-solution with the mixed-precision
DSGESV method (FP32 factorization whose trailing updates run on the BF16
tensor cores as split-BF16x3 products, FP64 residual / update / convergence
test on the GPU) against the plain FP64 GPU DGESV, at FP64 backward error.

One step = one DSGESV solve of the n=32768, nrhs=1 system
A = Q1 diag(s) Q2^T (Qi products of 64 Householder reflectors, s geometric
from 1 to 1/kappa, kappa=1e6), b = A x_true, with A and b resident in HBM
(8.6 GB of input, far larger than the 129 MB L2, so no flush is needed).
`e2e` measures the same solve through the LAPACK Fortran ABI (dsgesv_) with
pinned host buffers, the host<->device copies inside the timed region.

Inputs are synthetic, drawn from numpy's PCG64 with a fixed seed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --workload batched|adjoint|update|leaf ...   (one configuration or kernel class alone)
    python bench.py --workload dsposv|zgetrf [--wn N]            (the Cholesky and complex rows, device memory)
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "n=32768 DGESV time-to-solution: mixed-prec+IR vs FP64 GPU at FP64 backward err"
EPS = 2.0 ** -53

# DRAM bytes (read + write) of one launch, as a fraction of the launch's
# algorithmic bytes, from one ncu capture of the same kernel on a smaller
# case (profiles/gemm_bf16x3_trailing_update_n8192.md: M = N = 7936, K = 256,
# 459.5 MB measured against 520.1 MB algorithmic).  The traffic grows with
# M*N like the algorithmic bytes, so the ratio carries to n = 32768.
TRAFFIC_RATIO = {
    "gemm_bf16x3": (459.5 / 520.1, "ncu dram__bytes_read.sum + dram__bytes_write.sum of gemm_bf16x3_kernel at "
                                   "M=N=7936 K=256, scaled by algorithmic bytes"),
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=32768)
    p.add_argument("--nrhs", type=int, default=1)
    p.add_argument("--kappa", type=float, default=1e6)
    p.add_argument("--seed", type=int, default=2)
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU DGESV comparison")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-sweep", action="store_true", help="skip the per-kappa records (1e2, 1e6, 1e10)")
    p.add_argument("--no-sub", action="store_true", help="skip the batched and adjoint records of the default run")
    p.add_argument("--cpu-n", type=int, default=4096, help="size of the CPU baseline sample")
    p.add_argument("--workload", default="dsgesv",
                   choices=["dsgesv", "batched", "adjoint", "update", "leaf", "dgetrf", "dsposv", "zgetrf"],
                   help="dsgesv: the headline n=32768 solve; batched: 20000 uneven systems in one launch")
    p.add_argument("--dtype", default="d", choices=["d", "s"], help="precision of the batched workload")
    p.add_argument("--wn", type=int, default=0, help="order of the dsposv / zgetrf workloads (0: 8192 / 4096)")
    p.add_argument("--batch", type=int, default=20000)
    p.add_argument("--fixed-n", type=int, default=0, help="batched: every system of this size (0: uniform 8..512)")
    p.add_argument("--m", type=int, default=8192, help="update / leaf: rows (update: M = N)")
    p.add_argument("--k", type=int, default=256, help="update: K; leaf: panel width")
    return p.parse_args()


# ------------------------------------------------------------------ inputs
def make_system(n, kappa, seed, nrhs, device):
    """Column-major A (torch view with stride (1, n)), B, x_true on `device`.
    A = Q1 diag(s) Q2^T with 64 + 64 Householder reflectors; the storage
    array M holds A^T row-major (= A column-major)."""
    import torch
    rng = np.random.default_rng(seed)
    v1 = torch.from_numpy(rng.standard_normal((64, n))).to(device)
    v2 = torch.from_numpy(rng.standard_normal((64, n))).to(device)
    xt = torch.from_numpy(rng.standard_normal((n, nrhs))).to(device)
    i = torch.arange(n, dtype=torch.float64, device=device)
    s = kappa ** (-(i / max(n - 1, 1)))
    M = torch.diag(s)
    del s
    for v in v1:                       # M <- M H(v)
        tau = 2.0 / torch.dot(v, v)
        M.addr_(M @ v, v, alpha=-tau)
    for v in v2:                       # M <- H(v) M
        tau = 2.0 / torch.dot(v, v)
        M.addr_(v, v @ M, alpha=-tau)
    A = M.t()                          # (n, n) column-major view of A
    B = A @ xt                         # b = A x_true in FP64
    Bc = torch.empty((nrhs, n), dtype=torch.float64, device=device).t()
    Bc.copy_(B)
    return M, A, Bc, xt


def backward_errors(A, X, B, n):
    """DGET08 ratio ||b-Ax||_inf/(||A||_inf ||x||_inf eps) and the scaled
    residual of the headline metric (the same divided by n), computed on the
    GPU in FP64."""
    import torch
    R = B - A @ X
    anrm = A.abs().sum(dim=1).max().item()
    out = 0.0
    for j in range(X.shape[1]):
        out = max(out, R[:, j].abs().max().item() / (anrm * X[:, j].abs().max().item() * EPS))
    return out, out / n


def load_peaks():
    """Roofline denominators: the measured copy bandwidth and BF16 GEMM
    throughput of this machine's GPUs when MEASURED_PEAKS.json is present, else
    the fallback figures of an earlier GB300 measurement (6.8 TB/s, 1.9
    PFLOP/s BF16 burst), labelled as such."""
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        with open(pk_path) as f:
            peaks = json.load(f)
        if "hbm_gbs" in peaks and "bf16_tflops" in peaks:
            return peaks, "of measured (MEASURED_PEAKS.json)"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "of fallback (no MEASURED_PEAKS.json)"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.out.flush()
        self.out.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.out.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU baseline
def cpu_baseline(n_target, n_sample, kappa, seed, reps=1):
    """The oracle's DSGESV (the C restatement of SRC/dsgesv.f with the
    reference BLAS loops, column-parallel over all host cores) on an
    n_sample system of the same construction; time scaled by
    (n_target / n_sample)^3."""
    import oracle
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    a, _, _, _ = oracle.config_dsgesv_matrix(n_sample, kappa, seed)
    xt = np.random.default_rng(seed).standard_normal((n_sample, 1))
    b = a @ xt
    oracle.lib()
    times = []
    it = None
    for _ in range(reps):
        t0 = time.perf_counter()
        _, _, x, it, info = oracle.dsgesv(a, b)
        times.append(time.perf_counter() - t0)
    t = min(times)
    scale = (n_target / n_sample) ** 3
    return {"value": t * scale, "unit": "s", "cores": int(os.environ.get("OMP_NUM_THREADS", threads)),
            "kind": "port",
            "sample": f"oracle DSGESV at n={n_sample} (iter={it}), {t:.3f} s measured, "
                      f"time scaled by (n/{n_sample})^3 = {scale:.0f}"}


# -------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world):
    import torch
    import lapack_gb300 as g

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    L = g.lib()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    n, nrhs = args.n, args.nrhs

    M, A, B, xt = make_system(n, args.kappa, args.seed, nrhs, dev)
    X = torch.empty((nrhs, n), dtype=torch.float64, device=dev).t()
    ipiv = torch.empty(n, dtype=torch.int32, device=dev)
    it = ctypes.c_int(0)
    info = ctypes.c_int(0)

    def solve():
        rc = L.gb300_dsgesv_dev(n, nrhs, ctypes.c_void_p(A.data_ptr()), n, ctypes.c_void_p(ipiv.data_ptr()),
                                ctypes.c_void_p(B.data_ptr()), n, ctypes.c_void_p(X.data_ptr()), n,
                                ctypes.byref(it), ctypes.byref(info), sp)
        if rc != 0:
            raise RuntimeError(f"gb300_dsgesv_dev status {rc}")
        if it.value < 0:
            raise RuntimeError(f"refinement fell back to FP64 (ITER={it.value}); A no longer resident")

    for _ in range(args.warmup):
        solve()
    torch.cuda.synchronize()

    # one more untimed step with every kernel class bracketed by events: the
    # per-class breakdown and the dominant class
    names = ["gemm_f64", "gemm_f32_ffma", "gemm_bf16x3", "panel", "laswp", "trsm", "trsv", "residual_f64", "other",
             "copy_h2d", "copy_d2h"]
    L.gb300_prof_mask.restype = ctypes.c_uint
    L.gb300_prof_mask.argtypes = [ctypes.c_uint]

    def read_prof(steps):
        out = {}
        for k, nm in enumerate(names):
            t_ms, fl, by, cnt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
            L.gb300_prof_read(k, ctypes.byref(t_ms), ctypes.byref(fl), ctypes.byref(by), ctypes.byref(cnt))
            if cnt.value:
                out[nm] = {"ms_per_step": t_ms.value / steps, "launches_per_step": cnt.value / steps,
                           "flops": fl.value / steps, "bytes": by.value / steps}
        return out

    L.gb300_prof_reset()
    L.gb300_prof_mask(0xFFFFFFFF)
    L.gb300_prof_enable(1)
    solve()
    torch.cuda.synchronize()
    L.gb300_prof_enable(0)
    breakdown = read_prof(1)
    L.gb300_prof_reset()
    # the roofline is reported for the BF16x3 trailing update, the dominant
    # arithmetic kernel; the class that takes most device time (the panel
    # on the look-ahead stream, latency-bound) is named beside it
    top_class = max(breakdown, key=lambda k: breakdown[k]["ms_per_step"]) if breakdown else None
    dom_name = "gemm_bf16x3" if "gemm_bf16x3" in breakdown else top_class

    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(dev.index)
    clocks.start()
    # inside the timed region only the dominant class carries events
    if dom_name is not None:
        L.gb300_prof_mask(1 << names.index(dom_name))
        L.gb300_prof_enable(1)
    launches0 = L.gb300_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    iters = []
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        solve()
        iters.append(it.value)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = L.gb300_launch_count() - launches0
    L.gb300_prof_enable(0)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = t.item()

    # the dominant class's event times recorded inside the timed region
    timed = read_prof(args.steps)
    L.gb300_prof_reset()
    L.gb300_prof_mask(0xFFFFFFFF)

    # accuracy of the last solve
    bwd, scaled = backward_errors(A, X, B, n)
    fwd = ((X - xt).abs().max() / xt.abs().max()).item()

    peaks, peak_label = load_peaks()
    L.gb300_probe_peak.restype = ctypes.c_double
    dfma_peak = L.gb300_probe_peak(0)
    ffma_peak = L.gb300_probe_peak(1)
    # FP64 tensor-core (DMMA) throughput beside DFMA: the FP64 update runs on
    # whichever of the two is faster on this part
    dmma_peaks = {"m8n8k4": L.gb300_probe_peak(2), "m16n8k16": L.gb300_probe_peak(3)}

    # dominant kernel of the step and its roofline
    dom = (dom_name, timed.get(dom_name, breakdown.get(dom_name))) if dom_name else (None, None)
    roof = None
    if dom[0] is not None:
        nm, d = dom
        per_launch_ms = d["ms_per_step"] / d["launches_per_step"]
        if nm == "gemm_bf16x3":
            # C -= A B with K = 256: 3 BF16 products (6K flop) per 8 bytes of
            # C read+written, 192 flop/B, below the BF16/HBM ridge (~286
            # flop/B), so the update is HBM-bound; the tensor fraction is
            # reported beside it.
            tpeak = float(peaks["bf16_tflops"])
            hbm = float(peaks["hbm_gbs"])
            secs = d["ms_per_step"] * 1e-3
            tens = 3.0 * d["flops"] / secs / 1e12
            intensity = 3.0 * d["flops"] / d["bytes"]
            ridge = tpeak * 1e12 / (hbm * 1e9)
            if intensity < ridge:
                achieved = d["bytes"] / secs / 1e9
                roof = {"bound": "hbm", "kernel": nm, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                        "frac": achieved / hbm, "peak_source": f"hbm_gbs, {peak_label}"}
            else:
                achieved = tens
                roof = {"bound": "tensor", "kernel": nm, "achieved": achieved, "peak": tpeak, "unit": "TFLOP/s",
                        "frac": achieved / tpeak, "peak_source": f"bf16_tflops (burst), {peak_label}"}
            roof.update({"work": "per trailing update: 4*(M*K + K*N + 2*M*N) bytes (fp32 A, B read; C read "
                                 "and written), 3 BF16 products x 2*M*N*K flop",
                         "intensity_flop_per_byte": intensity, "ridge_flop_per_byte": ridge,
                         "tensor_tflops": tens, "tensor_frac": tens / tpeak})
        elif nm in ("gemm_f32_ffma", "gemm_f64", "panel", "trsm", "residual_f64"):
            peak = ffma_peak if nm != "gemm_f64" and nm != "residual_f64" else dfma_peak
            achieved = d["flops"] / (d["ms_per_step"] * 1e-3) / 1e12 if d["flops"] else 0.0
            roof = {"bound": "fp32-fma" if peak == ffma_peak else "fp64-fma", "kernel": nm, "achieved": achieved,
                    "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                    "peak_source": "gb300_probe_peak FMA loop measured in this run"}
        else:
            hbm = float(peaks["hbm_gbs"])
            achieved = d["bytes"] / (d["ms_per_step"] * 1e-3) / 1e9
            roof = {"bound": "hbm", "kernel": nm, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                    "frac": achieved / hbm, "peak_source": f"hbm_gbs, {peak_label}"}
        roof["per_launch_ms"] = per_launch_ms
        roof["traffic"] = None
        if nm in TRAFFIC_RATIO and d["bytes"]:
            ratio, src = TRAFFIC_RATIO[nm]
            roof["traffic"] = ratio * d["bytes"] / d["launches_per_step"]
            roof["traffic_unit"] = "bytes per launch"
            roof["traffic_source"] = src

    result = {
        "metric": METRIC, "value": ms * 1e-3, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/bf16x3 factor + f64 refine",
        "data": "synthetic",
        "config": {"workload": f"DSGESV n={n} nrhs={nrhs} kappa={args.kappa:g}: A=Q1 diag(s) Q2^T "
                               f"(64+64 Householder reflectors, s geometric 1..1/kappa), b=A x_true, "
                               f"inputs resident in HBM", "n": n, "nrhs": nrhs, "kappa": args.kappa,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs 8.6 GB >> 129 MB L2; no flush needed",
                   "mixed_mode": "bf16x3" if g.get_option("mixed") == 0 else "fp32-ffma",
                   "nb32": g.get_option("nb32"), "nb64": g.get_option("nb64"),
                   "lookahead": g.get_option("lookahead")},
        "iter": iters[-1], "backward_error_dget08": bwd, "scaled_residual": scaled, "forward_error": fwd,
        "dsgesv_stopping_test_met": bool(bwd < n ** 0.5),
        "kernel_ms_per_step": {k: v["ms_per_step"] for k, v in breakdown.items()},
        "kernel_launches_per_step": {k: v["launches_per_step"] for k, v in breakdown.items()},
        "roofline": roof, "gpu_launches": launches,
        "top_device_time_class": top_class,
        "panel_us_per_column": (breakdown["panel"]["ms_per_step"] * 1e3 / n) if "panel" in breakdown else None,
        "clocks": clk, "peaks_measured": {"dfma_tflops": dfma_peak, "ffma_tflops": ffma_peak,
                                          "dmma_tflops": dmma_peaks,
                                          "hbm_gbs": peaks.get("hbm_gbs"), "bf16_tflops": peaks.get("bf16_tflops"),
                                          "hbm_and_bf16_source": peak_label},
    }

    if not args.no_e2e:
        hA = torch.empty_like(M, device="cpu").pin_memory()
        hA.copy_(M)
        hB = torch.empty((nrhs, n), dtype=torch.float64).pin_memory()
        hB.copy_(B.t())
        hX = torch.empty((nrhs, n), dtype=torch.float64).pin_memory()
        hIp = torch.empty(n, dtype=torch.int32).pin_memory()
        work = np.zeros(1)
        swork = np.zeros(1, dtype=np.float32)
        ci = lambda v: ctypes.byref(ctypes.c_int(v))

        def e2e_step():
            L.dsgesv_(ci(n), ci(nrhs), ctypes.c_void_p(hA.data_ptr()), ci(n), ctypes.c_void_p(hIp.data_ptr()),
                      ctypes.c_void_p(hB.data_ptr()), ci(n), ctypes.c_void_p(hX.data_ptr()), ci(n),
                      work.ctypes.data_as(ctypes.c_void_p), swork.ctypes.data_as(ctypes.c_void_p),
                      ctypes.byref(it), ctypes.byref(info))
        def plain_copy_rates(k):
            # the host->device rate of the same pinned bytes by a plain copy:
            # the link's rate at that moment, which varies with the host
            rates = []
            for _ in range(k):
                c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                c0.record(stream)
                dst.copy_(hA, non_blocking=True)
                c1.record(stream)
                torch.cuda.synchronize()
                rates.append(8.0 * n * n / (c0.elapsed_time(c1) * 1e-3) / 1e9)
            return rates

        dst = torch.empty_like(M)
        e2e_step()
        torch.cuda.synchronize()
        before = plain_copy_rates(3)
        # each call with its copies bracketed by events: the split of the
        # end-to-end time into host->device copy, device work and device->host
        t_steps, splits = [], []
        L.gb300_prof_mask((1 << 9) | (1 << 10))
        for _ in range(max(3, min(args.steps, 5))):
            L.gb300_prof_reset()
            L.gb300_prof_enable(1)
            t0 = time.perf_counter()
            e2e_step()
            t_steps.append(time.perf_counter() - t0)
            L.gb300_prof_enable(0)
            sp_ = {}
            for k, nm in ((9, "h2d"), (10, "d2h")):
                t_ms, fl, by, cnt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
                L.gb300_prof_read(k, ctypes.byref(t_ms), ctypes.byref(fl), ctypes.byref(by), ctypes.byref(cnt))
                sp_[nm + "_s"] = t_ms.value * 1e-3
                sp_[nm + "_gbs"] = by.value / max(t_ms.value * 1e-3, 1e-12) / 1e9
            sp_["rest_s"] = t_steps[-1] - sp_["h2d_s"] - sp_["d2h_s"]
            splits.append(sp_)
        L.gb300_prof_reset()
        L.gb300_prof_mask(0xFFFFFFFF)
        after = plain_copy_rates(3)
        del dst
        t_e2e = statistics.median(t_steps)
        mid = t_steps.index(sorted(t_steps)[len(t_steps) // 2])
        split = dict(splits[mid])
        split["per_call"] = splits
        split["plain_copy_rates_gbs_before"] = before
        split["plain_copy_rates_gbs_after"] = after
        result["e2e"] = {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": 8 * n * n + 8 * n * nrhs,
                         "d2h_bytes_per_step": 8 * n * nrhs + 4 * n,
                         "path": "dsgesv_ (LAPACK Fortran ABI) on pinned host buffers, copies inside the call",
                         "steps_s": t_steps, "statistic": "median", "split_median_call": split}
        del hA, hB, hX
    # ---- plain FP64 GPU DGESV on the same system (the comparison arm)
    if not args.no_fp64:
        Ad = torch.empty_like(M)
        Ad.copy_(M)
        Ac = Ad.t()
        Xd = torch.empty((nrhs, n), dtype=torch.float64, device=dev).t()
        Xd.copy_(B)
        # warm the FP64 kernels on a small system first
        w = g.colmajor_empty(512, 512, torch.float64)
        w.copy_(torch.rand(512, 512, dtype=torch.float64, device=dev) + 4 * torch.eye(512, dtype=torch.float64,
                                                                                      device=dev))
        g.getrf_dev(w, torch.empty(512, dtype=torch.int32, device=dev))
        del w
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        rc = L.gb300_dgesv_dev(n, nrhs, ctypes.c_void_p(Ac.data_ptr()), n, ctypes.c_void_p(ipiv.data_ptr()),
                               ctypes.c_void_p(Xd.data_ptr()), n, ctypes.byref(info), sp)
        f1.record(stream)
        torch.cuda.synchronize()
        t64 = f0.elapsed_time(f1) * 1e-3
        bwd64, sc64 = backward_errors(A, Xd, B, n)
        result["fp64_gpu"] = {"seconds": t64, "status": rc, "info": info.value,
                              "tflops": (2.0 / 3.0) * n ** 3 / t64 / 1e12,
                              "frac_of_dfma_peak": (2.0 / 3.0) * n ** 3 / t64 / 1e12 / dfma_peak,
                              "backward_error_dget08": bwd64, "scaled_residual": sc64,
                              "forward_error": ((Xd - xt).abs().max() / xt.abs().max()).item()}
        result["speedup_vs_fp64_gpu"] = t64 / (ms * 1e-3)
        # the mixed solve's scaled residual against the FP64 GPU DGESV's on the
        # same system (the spec criterion), and separately DSGESV's own
        # stopping test ||r_i|| < ||x_i|| ||A|| eps sqrt(n) (SRC/dsgesv.f:337-342)
        result["backward_error_at_or_below_fp64"] = bool(scaled <= sc64)
        result["scaled_residual_ratio_mixed_over_fp64"] = scaled / sc64 if sc64 > 0 else None
        result["forward_error_vs_fp64_solve"] = ((X - Xd).abs().max() / Xd.abs().max()).item()
        fp64_headline = {"seconds": t64, "scaled_residual": sc64, "backward_error_dget08": bwd64,
                         "forward_error": result["fp64_gpu"]["forward_error"], "X": Xd}
        del Ad, Ac
        torch.cuda.empty_cache()

    # ---- accuracy and time-to-solution per condition number: the headline
    # system (kappa = 1e6) from above, then kappa = 1e2 and 1e10 solved once
    # each by the mixed driver and by the plain FP64 GPU DGESV.  At 1e10 the
    # refinement is expected to stop after 30 iterations (ITER = -31) and
    # fall back to the FP64 factorization, which is part of its time.
    if not args.no_sweep and not args.no_fp64:
        per = {}
        head = {"mixed_seconds": ms * 1e-3, "iter": iters[-1], "backward_error_dget08": bwd,
                "scaled_residual": scaled, "forward_error_vs_x_true": fwd,
                "forward_error_vs_fp64_solve": result["forward_error_vs_fp64_solve"],
                "dsgesv_stopping_test_met": bool(bwd < n ** 0.5),
                "fp64_seconds": fp64_headline["seconds"], "fp64_scaled_residual": fp64_headline["scaled_residual"],
                "fp64_backward_error_dget08": fp64_headline["backward_error_dget08"],
                "fp64_forward_error_vs_x_true": fp64_headline["forward_error"],
                "scaled_residual_at_or_below_fp64": bool(scaled <= fp64_headline["scaled_residual"]),
                "speedup_vs_fp64_gpu": fp64_headline["seconds"] / (ms * 1e-3)}
        per[f"{args.kappa:g}"] = head
        del fp64_headline
        for kap in (1e2, 1e6, 1e10):
            if f"{kap:g}" in per:
                continue
            del M, A, B
            torch.cuda.empty_cache()
            M, A, B, xt = make_system(n, kap, args.seed, nrhs, dev)
            per[f"{kap:g}"] = solve_once_both(L, g, M, A, B, xt, n, nrhs, ipiv, dev, stream, sp)
            if per[f"{kap:g}"]["iter"] > 0 and not per[f"{kap:g}"]["forward_error_vs_x_true"] < 1.0:
                # the refinement overflowed and DSGESV's stopping test passed
                # the NaN residual (SRC/dsgesv.f:384-389); the same system with
                # the library's NaN guard, which sends it to the FP64 solve
                old_guard = g.set_option("ir_nan_guard", 1)
                try:
                    per[f"{kap:g}"]["with_ir_nan_guard"] = solve_once_both(L, g, M, A, B, xt, n, nrhs, ipiv, dev,
                                                                           stream, sp, fp64=False)
                finally:
                    g.set_option("ir_nan_guard", old_guard)
        result["per_kappa"] = per
    return result


def solve_once_both(L, g, M, A, B, xt, n, nrhs, ipiv, dev, stream, sp, fp64=True):
    """One mixed DSGESV and (fp64=True) one plain FP64 DGESV of the same
    system, each on its own copy of A, timed with CUDA events on the
    launching stream, with their accuracy measures."""
    import torch
    it, info = ctypes.c_int(0), ctypes.c_int(0)
    X = torch.empty((nrhs, n), dtype=torch.float64, device=dev).t()
    Aw = M.clone()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    rc = L.gb300_dsgesv_dev(n, nrhs, ctypes.c_void_p(Aw.t().data_ptr()), n, ctypes.c_void_p(ipiv.data_ptr()),
                            ctypes.c_void_p(B.data_ptr()), n, ctypes.c_void_p(X.data_ptr()), n,
                            ctypes.byref(it), ctypes.byref(info), sp)
    e1.record(stream)
    torch.cuda.synchronize()
    t_mixed = e0.elapsed_time(e1) * 1e-3
    iter_mixed, info_mixed = it.value, info.value
    bw, sc = backward_errors(A, X, B, n)
    if not fp64:
        out = {"mixed_seconds": t_mixed, "status": rc, "iter": iter_mixed, "info": info_mixed,
               "backward_error_dget08": bw, "scaled_residual": sc,
               "forward_error_vs_x_true": ((X - xt).abs().max() / xt.abs().max()).item(),
               "dsgesv_stopping_test_met": bool(bw < n ** 0.5)}
        del Aw, X
        torch.cuda.empty_cache()
        return out
    Aw.copy_(M)
    Xd = torch.empty((nrhs, n), dtype=torch.float64, device=dev).t()
    Xd.copy_(B)
    torch.cuda.synchronize()
    e0.record(stream)
    rc64 = L.gb300_dgesv_dev(n, nrhs, ctypes.c_void_p(Aw.t().data_ptr()), n, ctypes.c_void_p(ipiv.data_ptr()),
                             ctypes.c_void_p(Xd.data_ptr()), n, ctypes.byref(info), sp)
    e1.record(stream)
    torch.cuda.synchronize()
    t64 = e0.elapsed_time(e1) * 1e-3
    bw64, sc64 = backward_errors(A, Xd, B, n)
    out = {"mixed_seconds": t_mixed, "status": rc, "iter": iter_mixed, "info": info_mixed,
           "backward_error_dget08": bw, "scaled_residual": sc,
           "forward_error_vs_x_true": ((X - xt).abs().max() / xt.abs().max()).item(),
           "forward_error_vs_fp64_solve": ((X - Xd).abs().max() / Xd.abs().max()).item(),
           "dsgesv_stopping_test_met": bool(bw < n ** 0.5),
           "fp64_seconds": t64, "fp64_status": rc64, "fp64_info": info.value, "fp64_scaled_residual": sc64,
           "fp64_backward_error_dget08": bw64,
           "fp64_forward_error_vs_x_true": ((Xd - xt).abs().max() / xt.abs().max()).item(),
           "scaled_residual_at_or_below_fp64": bool(sc <= sc64),
           "speedup_vs_fp64_gpu": t64 / t_mixed}
    del Aw, X, Xd
    torch.cuda.empty_cache()
    return out


def run_batched(args, rank=0, world=1):
    """20000 independent systems, n uniform in [8, 512] (seeded), nrhs in
    {1, 2, 4}, entries N(0,1) with n*I added to every other system, solved in
    one persistent launch captured in a CUDA graph.  One step = one graph
    replay over the whole batch (inputs restored between steps, outside the
    timed region).  Under torchrun the batch is partitioned over the ranks by
    LU cost (lapack_gb300.shard), each rank solving its share with no
    collective on the data path; the step time is the maximum over ranks."""
    import torch
    import lapack_gb300 as g
    from lapack_gb300 import autotune
    autotune.load()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    L = g.lib()
    dtype = torch.float64 if args.dtype == "d" else torch.float32
    es = 8 if args.dtype == "d" else 4
    rng = np.random.default_rng(args.seed)
    ns = rng.integers(8, 513, args.batch).astype(np.int64)
    if args.fixed_n > 0:
        ns[:] = args.fixed_n
    nrhs = rng.choice([1, 2, 4], args.batch).astype(np.int64)
    glob = np.arange(args.batch)                   # global system index of each local system
    if world > 1:
        from lapack_gb300 import shard
        glob = shard.partition_by_cost(ns, nrhs, world)[rank]
        ns, nrhs = ns[glob], nrhs[glob]
    batch = len(ns)
    aoff = np.concatenate([[0], np.cumsum(ns * ns)])
    boff = np.concatenate([[0], np.cumsum(ns * nrhs)])
    poff = np.concatenate([[0], np.cumsum(ns)])
    gen = torch.Generator(device=dev).manual_seed(args.seed)
    A = torch.randn(int(aoff[-1]), dtype=dtype, device=dev, generator=gen)
    B = torch.randn(int(boff[-1]), dtype=dtype, device=dev, generator=gen)
    # n*I on every other system's diagonal
    shifted = [i for i in range(batch) if glob[i] % 2 == 0]
    diag = np.concatenate([aoff[i] + np.arange(ns[i]) * (ns[i] + 1) for i in shifted])
    vals = np.concatenate([np.full(ns[i], float(ns[i])) for i in shifted])
    A.index_add_(0, torch.from_numpy(diag).to(dev), torch.from_numpy(vals).to(dev, dtype))
    A0, B0 = A.clone(), B.clone()
    ipiv = torch.zeros(int(poff[-1]), dtype=torch.int32, device=dev)
    info = torch.zeros(batch, dtype=torch.int32, device=dev)
    d_n = torch.from_numpy(ns.astype(np.int32)).to(dev)
    d_r = torch.from_numpy(nrhs.astype(np.int32)).to(dev)
    Ap = torch.from_numpy((A.data_ptr() + aoff[:-1] * es).astype(np.int64)).to(dev)
    Bp = torch.from_numpy((B.data_ptr() + boff[:-1] * es).astype(np.int64)).to(dev)
    Pp = torch.from_numpy((ipiv.data_ptr() + poff[:-1] * 4).astype(np.int64)).to(dev)
    fn = L.gb300_dgesv_vbatched_dev if args.dtype == "d" else L.gb300_sgesv_vbatched_dev
    vp = lambda t: ctypes.c_void_p(t.data_ptr())

    def launch(stream):
        rc = fn(batch, vp(d_n), vp(d_r), vp(Ap), vp(d_n), vp(Pp), vp(Bp), vp(d_n), vp(info),
                ctypes.c_void_p(stream.cuda_stream))
        if rc:
            raise RuntimeError(f"batched solve status {rc}")

    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        launch(s)                      # warm-up (kernel attributes, pool)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    A.copy_(A0)
    B.copy_(B0)
    torch.cuda.synchronize()
    # the library kernels one replay runs: those the captured call launched
    # (a replay itself passes no launch through the library's counter)
    launches_cap0 = L.gb300_launch_count()
    with torch.cuda.stream(s):
        graph.capture_begin()
        launch(s)
        graph.capture_end()
    launches_per_replay = L.gb300_launch_count() - launches_cap0
    times = []
    clocks = ClockSampler(dev.index)
    clocks.start()
    for it in range(args.warmup + args.steps):
        A.copy_(A0)
        B.copy_(B0)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        graph.replay()
        e1.record()
        torch.cuda.synchronize()
        if it >= args.warmup:
            times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    ms = sum(times) / len(times)
    flops = float(np.sum(2.0 / 3.0 * ns.astype(np.float64) ** 3 + 2.0 * ns ** 2 * nrhs))
    bytes_ = float(np.sum(es * (2.0 * ns * ns + 2.0 * ns * nrhs) + 4.0 * ns))
    info_nonzero = int((info != 0).sum().item())
    if world > 1:
        # whole-job figures: the slowest rank's time, the work of all ranks
        red = torch.tensor([ms, 0.0, 0.0, 0.0], dtype=torch.float64, device=dev)
        tot = torch.tensor([0.0, flops, bytes_, float(info_nonzero)], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(red, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(tot, op=torch.distributed.ReduceOp.SUM)
        ms, flops, bytes_, info_nonzero = float(red[0]), float(tot[1]), float(tot[2]), int(tot[3])
    peaks, peak_label = load_peaks()
    L.gb300_probe_peak.restype = ctypes.c_double
    fma_peak = L.gb300_probe_peak(0 if args.dtype == "d" else 1)
    hbm = float(peaks["hbm_gbs"])
    # residual spot check of a few systems
    hA, hB = A0.cpu().numpy(), B0.cpu().numpy()
    X = B.cpu().numpy()
    worst = 0.0
    for i in list(range(0, batch, max(1, batch // 8))):
        n, r = int(ns[i]), int(nrhs[i])
        a = hA[aoff[i]:aoff[i + 1]].reshape(n, n).T.astype(np.float64)
        b = hB[boff[i]:boff[i + 1]].reshape(r, n).T.astype(np.float64)
        x = X[boff[i]:boff[i + 1]].reshape(r, n).T.astype(np.float64)
        res = np.abs(b - a @ x).max() / (np.abs(a).sum(1).max() * np.abs(x).max() * n * (2.0 ** -53 if args.dtype == "d" else 2.0 ** -24))
        worst = max(worst, res)
    return {
        "metric": f"batched uneven {'D' if args.dtype == 'd' else 'S'}GESV: {args.batch} systems, n in [8,512], nrhs in {{1,2,4}}, one persistent launch",
        "value": ms * 1e-3, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": False, "scaling": "strong", "dtype": "f64" if args.dtype == "d" else "f32",
        "data": "synthetic",
        "config": {"workload": "batched uneven solves in one CUDA-graph-captured persistent launch", "batch": args.batch,
                   "parallelism": (f"systems partitioned by LU cost over {world} ranks, no collective"
                                   if world > 1 else "single GPU"),
                   "nb_table": g.vbatched_nb(0 if args.dtype == "d" else 1),
                   "l2": f"inputs {bytes_ / 2e9:.1f} GB >> L2"},
        "gflops": flops / ms / 1e6, "fma_peak_tflops": fma_peak, "frac_of_fma_peak": flops / ms / 1e9 / (fma_peak * world),
        "hbm_gbs": bytes_ / ms / 1e6, "frac_of_hbm": bytes_ / ms / 1e6 / (hbm * world), "algorithmic_bytes": bytes_,
        "algorithmic_flops": flops, "info_nonzero": info_nonzero, "worst_scaled_residual": worst,
        "gpu_launches": launches_per_replay, "gpu_launches_note": "library kernels per graph replay, counted at capture",
        "clocks": clk,
    }


def run_adjoint(args):
    """The differentiable batched solve: 64 systems of n = 2048,
    A = N(0,1)/sqrt(n) + I, B and gX of 8 columns.  One step = the adjoint of
    the whole batch (gB = A^{-T} gX by the transposed solve on the stored
    factors, gA = -gB X^T written in full: 2 GiB), factors resident."""
    import torch
    import lapack_gb300 as g
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    L = g.lib()
    batch, n, nrhs = 64, 2048, 8
    gen = torch.Generator(device=dev).manual_seed(args.seed)
    LU = torch.randn(batch, n, n, dtype=torch.float64, device=dev, generator=gen) / n ** 0.5
    LU += torch.eye(n, dtype=torch.float64, device=dev)
    X = torch.randn(batch, nrhs, n, dtype=torch.float64, device=dev, generator=gen)
    GX = torch.randn(batch, nrhs, n, dtype=torch.float64, device=dev, generator=gen)
    ip = torch.empty(batch, n, dtype=torch.int32, device=dev)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    info = ctypes.c_int(0)
    vp = ctypes.c_void_p
    t0 = time.perf_counter()
    for k in range(batch):
        L.gb300_dgesv_dev(n, nrhs, vp(LU[k].data_ptr()), n, vp(ip[k].data_ptr()), vp(X[k].data_ptr()), n,
                          ctypes.byref(info), s)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    GB = torch.empty_like(GX)
    GA = torch.empty_like(LU)

    def step():
        rc = L.gb300_dgesv_adjoint_batched_dev(batch, n, nrhs, vp(LU.data_ptr()), n * n, vp(ip.data_ptr()), n,
                                               vp(X.data_ptr()), n * nrhs, vp(GX.data_ptr()), n * nrhs,
                                               vp(GB.data_ptr()), n * nrhs, vp(GA.data_ptr()), n * n, s)
        if rc:
            raise RuntimeError(f"adjoint status {rc}")
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    L.gb300_prof_reset()
    L.gb300_prof_enable(1)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    L.gb300_prof_enable(0)
    ms = e0.elapsed_time(e1) / args.steps
    parts = {}
    for k, nm in enumerate(["gemm_f64", "gemm_f32_ffma", "gemm_bf16x3", "panel", "laswp", "trsm", "trsv",
                            "residual_f64", "ipiv_replay_and_gA"]):
        t_ms, fl, by, cnt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        L.gb300_prof_read(k, ctypes.byref(t_ms), ctypes.byref(fl), ctypes.byref(by), ctypes.byref(cnt))
        if cnt.value:
            parts[nm] = {"ms_per_step": t_ms.value / args.steps, "gbs": by.value / max(t_ms.value, 1e-9) / 1e6}
    L.gb300_prof_reset()
    peaks, peak_label = load_peaks()
    hbm = float(peaks["hbm_gbs"])
    bytes_ = batch * (8.0 * n * n * 2 + 8.0 * n * nrhs * 4)     # LU read by the solves + gA written + vectors
    # both halves do 2*n^2*nrhs flop per system (the two triangular solves
    # together, and gA = -gB X^T): 2 flop per byte of LU read or gA written,
    # above the FP64/HBM ridge, so the step is FP64-FMA-bound
    flops = batch * 4.0 * n * n * nrhs
    L.gb300_probe_peak.restype = ctypes.c_double
    dfma = L.gb300_probe_peak(0)
    tf = flops / (ms * 1e-3) / 1e12
    return {"metric": "adjoint of X = A^{-1}B: 64 systems n=2048 nrhs=8 (gB by transposed solve, gA = -gB X^T)",
            "value": ms * 1e-3, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": False, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "adjoint batch 64 x n=2048 x nrhs=8, factors resident", "forward_s": t_fwd},
            "kernels": parts, "algorithmic_bytes": bytes_, "hbm_gbs": bytes_ / ms / 1e6,
            "frac_of_hbm": bytes_ / ms / 1e6 / hbm,
            "roofline": {"bound": "fp64-fma", "achieved": tf, "peak": dfma, "unit": "TFLOP/s", "frac": tf / dfma,
                         "peak_source": "gb300_probe_peak FP64 FMA loop measured in this run",
                         "work": "4*n^2*nrhs flop per system"}}


def run_widened(args):
    """The widened rows on device memory, one call per step, the inputs
    restored before each call outside the timed region: 'dsposv' is
    DSPOSV('L') of the SPD system A = X X^T/64 + I (X: 64 columns uniform in
    [-1, 1]), b = A*1; 'zgetrf' is ZGETRF of a matrix whose real and
    imaginary parts are uniform in [-1, 1].  Times are CUDA events on the
    launching stream; the value is the median over the steps."""
    import torch
    import lapack_gb300 as g
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    L = g.lib()
    vp = ctypes.c_void_p
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    gen = torch.Generator(device=dev).manual_seed(args.seed)
    it, info = ctypes.c_int(0), ctypes.c_int(0)
    if args.workload == "dsposv":
        n = args.wn or 8192
        Xr = torch.rand(n, 64, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
        A0 = Xr @ Xr.t() / 64 + torch.eye(n, dtype=torch.float64, device=dev)
        B = A0.sum(1).contiguous()
        X = torch.empty_like(B)
        A = torch.empty_like(A0)

        def call():
            return L.gb300_dsposv_dev(ctypes.c_char(b"L"), n, 1, vp(A.data_ptr()), n, vp(B.data_ptr()), n,
                                      vp(X.data_ptr()), n, ctypes.byref(it), ctypes.byref(info), s)
        flops, metric, dtype = n ** 3 / 3.0, f"DSPOSV('L') n={n} nrhs=1 on device memory", "f32 factor + f64 refine"
    else:
        n = args.wn or 4096
        A0 = torch.complex(torch.rand(n, n, dtype=torch.float64, device=dev, generator=gen) * 2 - 1,
                           torch.rand(n, n, dtype=torch.float64, device=dev, generator=gen) * 2 - 1)
        A = torch.empty_like(A0)
        ip = torch.empty(n, dtype=torch.int32, device=dev)

        def call():
            return L.gb300_zgetrf_dev(n, n, vp(A.data_ptr()), n, vp(ip.data_ptr()), ctypes.byref(info), s)
        flops, metric, dtype = 8.0 / 3.0 * n ** 3, f"ZGETRF n={n} on device memory", "c128"
    times = []
    for k in range(args.warmup + args.steps):
        A.copy_(A0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = call()
        e1.record()
        torch.cuda.synchronize()
        if rc:
            raise RuntimeError(f"{args.workload} status {rc}")
        if k >= args.warmup:
            times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    out = {"metric": metric, "value": ms * 1e-3, "unit": "s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "dtype": dtype,
           "data": "synthetic", "config": {"workload": args.workload, "n": n, "exact": g.get_option("exact")},
           "tflops": flops / ms / 1e9, "info": info.value}
    if args.workload == "dsposv":
        out["iter"] = it.value
        out["max_abs_error_vs_ones"] = (X - 1).abs().max().item()
    return out


def run_kernel_case(args):
    """One kernel class alone, for timing and profiling: 'update' is the
    BF16x3 trailing update C -= A B of an M x M matrix with K = k
    (gb300_sgemm_update_dev, mode 0); 'leaf' is the FP32 LU of one m x k
    panel (gb300_sgetrf_dev on the panel: one cluster leaf for k up to the
    leaf width).  Four untimed calls, then `steps` calls timed with CUDA
    events on the launching stream."""
    import torch
    import lapack_gb300 as g
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    L = g.lib()
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    gen = torch.Generator(device=dev).manual_seed(args.seed)
    m, k = args.m, args.k
    if args.workload == "update":
        A = g.colmajor_empty(m, k, torch.float32)
        A.copy_(torch.randn(m, k, device=dev, generator=gen))
        B = g.colmajor_empty(k, m, torch.float32)
        B.copy_(torch.randn(k, m, device=dev, generator=gen))
        C = g.colmajor_empty(m, m, torch.float32)
        C.copy_(torch.randn(m, m, device=dev, generator=gen))

        def call():
            rc = L.gb300_sgemm_update_dev(0, m, m, k, ctypes.c_void_p(A.data_ptr()), m, ctypes.c_void_p(B.data_ptr()),
                                          k, ctypes.c_void_p(C.data_ptr()), m, sp)
            if rc:
                raise RuntimeError(f"update status {rc}")
        work = {"bytes": 4.0 * (m * k + k * m + 2.0 * m * m), "flops": 2.0 * m * m * k}
    elif args.workload == "dgetrf":
        A0 = g.colmajor_empty(m, m, torch.float64)
        A0.copy_(torch.rand(m, m, dtype=torch.float64, device=dev, generator=gen) * 2 - 1)
        A = A0.clone()
        ip = torch.empty(m, dtype=torch.int32, device=dev)

        def call():
            A.copy_(A0)
            g.getrf_dev(A, ip)
        work = {"bytes": 2.0 * 8.0 * m * m, "flops": 2.0 / 3.0 * m ** 3}
    else:
        P0 = g.colmajor_empty(m, k, torch.float32)
        P0.copy_(torch.rand(m, k, device=dev, generator=gen) * 2 - 1)
        P = P0.clone()
        ip = torch.empty(k, dtype=torch.int32, device=dev)

        def call():
            P.copy_(P0)
            g.getrf_dev(P, ip)
        work = {"bytes": 2.0 * 4.0 * m * k, "flops": float(m) * k * k}
    for _ in range(4):
        call()
    torch.cuda.synchronize()
    # the panel class (the leaf kernel alone) carries events in the leaf case
    if args.workload == "leaf":
        L.gb300_prof_reset()
        L.gb300_prof_mask(1 << 3)
        L.gb300_prof_enable(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(args.steps):
        call()
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    ms_call = ms
    if args.workload == "leaf":
        L.gb300_prof_enable(0)
        t_ms, fl, by, cnt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        L.gb300_prof_read(3, ctypes.byref(t_ms), ctypes.byref(fl), ctypes.byref(by), ctypes.byref(cnt))
        L.gb300_prof_reset()
        L.gb300_prof_mask(0xFFFFFFFF)
        ms = t_ms.value / max(cnt.value, 1)
    out = {"workload": args.workload, "m": m, "k": k,
           ("ms_per_leaf_kernel" if args.workload == "leaf" else "ms_per_call"): ms,
           "algorithmic_gbs": work["bytes"] / ms / 1e6, "tflops": work["flops"] / ms / 1e9,
           "options": {o: g.get_option(o) for o in ("gemm_ws", "gemm_tiles", "cluster_panel")}}
    if args.workload == "update":
        out["tensor_tflops_3_products"] = 3.0 * work["flops"] / ms / 1e9
    elif args.workload == "leaf":
        # the latency floor of one leaf column: the skeleton of its exchange
        # (two CTA barriers around a cluster-wide exchange) on one cluster
        L.gb300_probe_cluster_exchange.restype = ctypes.c_double
        L.gb300_probe_cluster_exchange.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        out["cluster_exchange_us_per_column"] = {
            f"{mode}_{ctas}": L.gb300_probe_cluster_exchange(ctas, 0 if mode == "push" else 1, 20000)
            for mode in ("push", "barrier") for ctas in (16, 8)}
        out["us_per_column"] = ms * 1e3 / k
        # the whole panel call: its leaves, the solves and updates between them
        out["ms_per_panel_call"] = ms_call
    return out


def main():
    args = parse()
    if args.workload in ("update", "leaf", "dgetrf"):
        print(json.dumps(run_kernel_case(args)))
        return
    if args.workload in ("dsposv", "zgetrf"):
        print(json.dumps(run_widened(args)))
        return
    if args.workload == "batched" and args.impl == "gb300":
        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        if world > 1:
            import torch
            torch.distributed.init_process_group("nccl")
        result = run_batched(args, rank, world)
        if rank == 0:
            print(json.dumps(result))
        if world > 1:
            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
        return
    if args.workload == "adjoint" and args.impl == "gb300":
        print(json.dumps(run_adjoint(args)))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        # the reference arm: the oracle port of the reference routines on the
        # host cores, rank 0 only
        if rank != 0:
            return
        samples = []
        for _ in range(args.warmup):
            cpu_baseline(args.n, args.cpu_n, args.kappa, args.seed)
        for _ in range(args.steps):
            samples.append(cpu_baseline(args.n, args.cpu_n, args.kappa, args.seed))
        v = statistics.median(s["value"] for s in samples)
        cb = dict(samples[0])
        cb["value"] = v
        print(json.dumps({
            "metric": METRIC, "impl": "reference", "value": v, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 factor + f64 refine", "data": "synthetic",
            "config": {"workload": f"DSGESV n={args.n} nrhs={args.nrhs} kappa={args.kappa:g} (CPU sample "
                                   f"n={args.cpu_n}, scaled by n^3)", "n": args.n, "kappa": args.kappa},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    result = run_gpu(args, rank, world)
    if not args.no_sub and world == 1:
        # the other configurations of the path, one record each beside the
        # headline: the batched uneven solves (FP32 and FP64) and the adjoint
        import torch
        torch.cuda.empty_cache()
        subs = {}
        for dt in ("s", "d"):
            a2 = argparse.Namespace(**vars(args))
            a2.dtype, a2.steps, a2.warmup = dt, 3, 2
            subs["batched_f32" if dt == "s" else "batched_f64"] = run_batched(a2, 0, 1)
            torch.cuda.empty_cache()
        a3 = argparse.Namespace(**vars(args))
        a3.steps, a3.warmup = 5, 2
        subs["adjoint"] = run_adjoint(a3)
        result["sub_workloads"] = subs
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(args.n, args.cpu_n, args.kappa, args.seed)
    if rank == 0:
        print(json.dumps(result))
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
