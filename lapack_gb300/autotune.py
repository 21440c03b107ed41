"""Autotuner for the batched uneven-size solver and the blocked LU.

Batched: for every 64-row size bucket (n in 1..64, 65..128, ..., 449..512)
and every candidate panel width, a synthetic batch of systems of that bucket
is solved in one launch and timed with CUDA events; the fastest width per
bucket becomes the table the persistent kernel reads
(gb300_vbatched_set_nb).  Blocked LU: the outer block size of the FP32
factorization in DSGESV's mode (BF16x3 updates; NB in 192..384 at
n = 32768, the DSGESV size) and of the FP64 one (NB in 64..256 at
n = 16384, the FP64 DGESV configuration's size); each the best of three
runs.

Results are written to autotune.json next to this file; `load()` installs
them (import of the package does this when the file exists).

    python -m lapack_gb300.autotune [--quick]
"""
import argparse
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "autotune.json")
CANDIDATES = {0: [8, 16], 1: [8, 16, 32]}      # per dtype code (0 double, 1 float): the panel capacities


def _time_batch(g, As, Bs, dtype, reps=3):
    import torch
    vb = g.VBatch(As, Bs, dtype)
    a0, b0 = vb.A.clone(), vb.B.clone()
    vb.launch()
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        vb.A.copy_(a0)
        vb.B.copy_(b0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        vb.launch()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def tune_batched(dtype_code, count=600, seed=0):
    import torch
    import lapack_gb300 as g
    dtype = torch.float64 if dtype_code == 0 else torch.float32
    ne = np.float64 if dtype_code == 0 else np.float32
    rng = np.random.default_rng(seed)
    table = list(g.vbatched_nb(dtype_code))
    timings = {}
    for b in range(8):
        lo, hi = 64 * b + 1, 64 * b + 64
        ns = rng.integers(max(lo, 2), hi + 1, count if b < 4 else count // 2)
        As = [(rng.standard_normal((n, n)) + n * np.eye(n)).astype(ne) for n in ns]
        Bs = [rng.standard_normal((n, 1)).astype(ne) for n in ns]
        res = {}
        for nb in CANDIDATES[dtype_code]:
            trial = list(table)
            trial[b] = nb
            g.set_vbatched_nb(dtype_code, trial)
            res[nb] = _time_batch(g, As, Bs, dtype)
        table[b] = min(res, key=res.get)
        timings[f"{lo}-{hi}"] = res
        g.set_vbatched_nb(dtype_code, table)
    return table, timings


def tune_getrf_nb(dtype_code, n, candidates, reps=3):
    import torch
    import lapack_gb300 as g
    dtype = torch.float64 if dtype_code == 0 else torch.float32
    key = "nb64" if dtype_code == 0 else "nb32"
    # the FP32 block size serves DSGESV's factorization: tune it in that
    # factorization's mode (BF16x3 trailing updates)
    old_mode = g.set_option("sgetrf", 0) if dtype_code == 1 else None
    A0 = g.colmajor_empty(n, n, dtype)
    A0.copy_(torch.rand(n, n, dtype=dtype, device="cuda") * 2 - 1)
    ip = torch.empty(n, dtype=torch.int32, device="cuda")
    res = {}
    for nb in candidates:
        g.set_option(key, nb)
        A = A0.clone()
        g.getrf_dev(A, ip)
        best_ms = float("inf")
        for _ in range(reps):          # the best of a few runs: one run can catch a slow clock
            A.copy_(A0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            g.getrf_dev(A, ip)
            e1.record()
            torch.cuda.synchronize()
            best_ms = min(best_ms, e0.elapsed_time(e1))
        res[nb] = best_ms
    best = min(res, key=res.get)
    g.set_option(key, best)
    if old_mode is not None:
        g.set_option("sgetrf", old_mode)
    return best, res


def load(path=TABLE):
    """Installs a saved table; returns it (or None)."""
    if not os.path.exists(path):
        return None
    import lapack_gb300 as g
    with open(path) as f:
        t = json.load(f)
    for code in (0, 1):
        tab = t.get("batched", {}).get(str(code))
        if tab:
            g.set_vbatched_nb(code, tab["table"])
    for key in ("nb64", "nb32"):
        if key in t.get("getrf", {}):
            g.set_option(key, int(t["getrf"][key]["best"]))
    return t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="fewer systems per bucket, no LU block sweep")
    ap.add_argument("--out", default=TABLE)
    args = ap.parse_args()
    out = {"batched": {}, "getrf": {}}
    for code in (0, 1):
        table, timings = tune_batched(code, count=150 if args.quick else 600)
        out["batched"][str(code)] = {"table": table, "ms": timings}
        print("batched", "double" if code == 0 else "float", table, flush=True)
    if not args.quick:
        # FP32: DSGESV's factorization at the headline size (n = 32768);
        # FP64: the FP64 DGESV configuration's size (n = 16384)
        best, res = tune_getrf_nb(1, 32768, [192, 256, 320, 384])
        out["getrf"]["nb32"] = {"n": 32768, "best": best, "ms": res}
        best, res = tune_getrf_nb(0, 16384, [64, 96, 128, 192, 256])
        out["getrf"]["nb64"] = {"n": 16384, "best": best, "ms": res}
        print("getrf", out["getrf"], flush=True)
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(args.out)


if __name__ == "__main__":
    main()
