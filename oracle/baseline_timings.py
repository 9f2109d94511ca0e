"""Baseline timings for the benchmark spec (test infrastructure, not the product).

Times, on the GPU machine:
  * the reference's own FP32 kernels (pcrGauss rows: `rest` is g), rebuilt for sm_103a from its sources
    (oracle/_ref cubins, launched by oracle/ref_kernels_runner.cpp with the
    reference launchers' grid / block / shared sizes), beside this project's
    kernels on the same inputs;
  * the gold CPU Thomas (oracle/gold.c, bit-identical to tridiagonal_gold.h)
    on 1 core and on every core, FP32 and FP64.

The reference kernels overwrite a, b, c, d, so every timed launch starts from
a fresh copy (the copy is outside the timed events).  Median of `reps`
launches.  Prints one JSON object per line.

    python oracle/baseline_timings.py [--reps 50] [--no-cpu]
"""
from __future__ import annotations

import argparse
import json
import statistics
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def time_reference(kind, n, m, rest, reps):
    import torch

    from oracle.gold import RefKernels
    from tridiagonalsolvers_gb300 import workloads

    rk = RefKernels()
    a, b, c, d = workloads.dominant(m, n, seed=workloads.SEEDS["c2"])
    src = [torch.from_numpy(v).cuda() for v in (a, b, c, d)]
    work = [torch.empty_like(t) for t in src]
    ping = [torch.empty_like(t) for t in src] if kind == "pcrGauss" else None
    x = torch.empty_like(src[0])
    times = []
    for r in range(reps + 3):
        for w, s in zip(work, src):
            w.copy_(s)
        e0, e1 = _events()
        e0.record()
        if kind == "pcrGauss":  # rest = g; the solution is left in d or its ping buffer
            rk.pcr_gauss(*work, *ping, n, m, rest, torch.cuda.current_stream().cuda_stream)
        else:
            rk.solve(kind, *work, x, n, m, rest, torch.cuda.current_stream().cuda_stream)
        e1.record()
        torch.cuda.synchronize()
        if r >= 3:
            times.append(e0.elapsed_time(e1))
    return statistics.median(times)


def time_ours(kind, n, m, rest, reps):
    import ctypes

    import torch

    from tridiagonalsolvers_gb300 import _lib, workloads

    L = _lib.lib()
    a, b, c, d = workloads.dominant(m, n, seed=workloads.SEEDS["c2"])
    t = [torch.from_numpy(v).cuda() for v in (a, b, c, d)]
    x = torch.empty_like(t[0])
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptrs = [v.data_ptr() for v in (*t, x)]
    fn = {"cr": lambda: L.tridi_cr_f32(*ptrs, n, m, sp), "pcr": lambda: L.tridi_pcr_f32(*ptrs, n, m, sp),
          "crpcr": lambda: L.tridi_crpcr_f32(*ptrs, n, m, rest, sp),
          "crNBC": lambda: L.tridi_cr_nbc_f32(*ptrs, n, m, sp),
          "crpcrNBC": lambda: L.tridi_crpcr_nbc_f32(*ptrs, n, m, rest, sp),
          "crNBC32": lambda: L.tridi_cr_nbc_f32(*ptrs, n, m, sp),
          "pcrGauss": lambda: L.tridi_pcr_thomas_f32(*ptrs, n, m, rest, sp)}[kind]
    times = []
    for r in range(reps + 3):
        e0, e1 = _events()
        e0.record()
        _lib.check(fn(), kind)
        e1.record()
        torch.cuda.synchronize()
        if r >= 3:
            times.append(e0.elapsed_time(e1))
    return statistics.median(times)


def gpu_rows(reps, peak):
    cases = []
    for n, m in ((512, 512), (256, 65536), (1024, 16384)):
        for kind in ("cr", "pcr", "crNBC", "crNBC32"):
            if kind == "pcr" and n > 1024:
                continue
            cases.append((kind, n, m, 0))
        rest = 2
        while rest <= n // 2:
            cases.append(("crpcr", n, m, rest))
            rest *= 2
        cases.append(("crpcrNBC", n, m, 32 if n >= 64 else 2))
        if n <= 1024:  # the reference's small pcrGauss path; g = 8 (exact there) and n/2 (at most 512)
            cases += [("pcrGauss", n, m, 8), ("pcrGauss", n, m, min(n // 2, 512))]
    for kind, n, m, rest in cases:
        row = {"kernel": kind, "n": n, "m": m, "rest": rest or None}
        for who, f in (("reference", time_reference), ("ours", time_ours)):
            try:
                ms = f(kind, n, m, rest, reps)
                gbs = 20.0 * n * m / (ms * 1e-3) / 1e9
                row[who] = {"ms": round(ms, 5), "unknowns_per_s": n * m / (ms * 1e-3), "gbs": round(gbs, 1),
                            "frac_of_hbm": round(gbs / peak, 4)}
            except Exception as e:  # a shape the kernel does not launch
                row[who] = {"error": str(e)[:120]}
        print(json.dumps(row), flush=True)


def cpu_rows():
    from oracle import gold
    from tridiagonalsolvers_gb300 import workloads

    lib = gold.gold_lib()
    cores = lib.gold_max_threads()
    for n, m in ((512, 512), (256, 8192), (1024, 2048)):
        for dtype in (np.float32, np.float64):
            a, b, c, d = (v.astype(dtype) for v in workloads.dominant(m, n, seed=workloads.SEEDS["c2"]))
            for threads in (1, cores):
                gold.serial_many(a[:8], b[:8], c[:8], d[:8], threads=threads)
                reps, t0 = 0, time.perf_counter()
                while time.perf_counter() - t0 < 1.0:
                    gold.serial_many(a, b, c, d, threads=threads)
                    reps += 1
                el = time.perf_counter() - t0
                print(json.dumps({"cpu_gold": "serial Thomas", "dtype": np.dtype(dtype).name, "n": n, "m": m,
                                  "threads": threads, "unknowns_per_s": reps * n * m / el}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=50)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-gpu", action="store_true")
    args = ap.parse_args()
    peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"] if (ROOT / "MEASURED_PEAKS.json").exists() else 6800.0
    if not args.no_gpu:
        gpu_rows(args.reps, peak)
    if not args.no_cpu:
        cpu_rows()


if __name__ == "__main__":
    main()
