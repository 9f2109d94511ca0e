"""Benchmark of the batched FP32 tridiagonal solve on GB300.

Workload (one "step"): one solve of the large fixed-size FP32 batch,
65536 independent systems x 256 unknowns, contiguous per-system layout,
seeded strictly diagonally dominant inputs (a, c ~ U[-1,1], a[0] = c[n-1] = 0,
b = |a|+|c|+U[1,2], d ~ U[-1,1]), solved by cyclic reduction (cr).  The
inputs (4 x 64 MiB) are larger than the 129 MB L2, so nothing is flushed
between steps.  Metric: unknowns solved per second; the roofline is the HBM
bandwidth at 20 algorithmic bytes per unknown (a, b, c, d read, x written).

Lines printed (rank 0, one JSON line):
  * value: device-resident throughput (CUDA events around K back-to-back
    steps on the launching stream, max over ranks);
  * e2e: the same through the reference-facing host-pointer launcher
    (tridi_dropin_solve_f32 = cr()), pinned host buffers (which the solver
    reads and writes in place over the host link), every byte's transfer
    inside the timed region;
  * roofline, cpu_baseline, clocks, per-kernel table (cr, crNBC, pcr, crpcr
    over its switch levels) for the same batch.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
  python bench.py --workload kernel --kernel pcr --system-size 256 --num-systems 65536 [--param P]

--impl reference times the reference's own CPU gold solver (the oracle's
restatement of tridiagonal_gold.h, bit-identical to it) on every host core,
on a bounded sample of the same workload.

--gpus N > 1 without a launcher's WORLD_SIZE re-runs this script under
torch.distributed.run with N ranks, one GPU each: N independent replicas
(weak scaling, no data-path collective), timed with a barrier on both sides
and the maximum over ranks.

Code under oracle/ runs in two reported-baseline legs only, never in the
timed region: cpu_baseline (and the --impl reference arm) time the gold
Thomas solver; reference_kernels times the reference's own CUDA kernels
rebuilt for sm_103a (oracle/_ref cubins through oracle/ref_kernels_runner.cpp)
on the same batch, beside each row of the per-kernel table.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

M, N = 65536, 256
BYTES_PER_UNKNOWN = 20  # a, b, c, d in + x out, FP32
METRIC = "unknowns/s"
WORKLOAD = "batched FP32 tridiagonal solve, 65536 systems x 256 unknowns, contiguous"


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def rel_residual64(a, b, c, d, x):
    """Per system ||d - T x||_2 / ||d||_2 in FP64, rows are systems (a[:, 0]
    and c[:, -1] ignored): the guard that a timed result solves its systems."""
    a, b, c, d, x = (np.asarray(v, np.float64) for v in (a, b, c, d, x))
    r = d - b * x
    r[:, 1:] -= a[:, 1:] * x[:, :-1]
    r[:, :-1] -= c[:, :-1] * x[:, 1:]
    return np.linalg.norm(r, axis=1) / np.maximum(np.linalg.norm(d, axis=1), 1e-300)


def profile_value(name: str, key: str):
    """A figure recorded in a committed ncu summary under profiles/ (None if absent)."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def profile_traffic():
    """dram bytes per launch of the headline kernel from the committed ncu summary."""
    return profile_value("cr_65536x256_ncu.md", "traffic_bytes_per_launch")


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            f = [v.strip() for v in line.split(",")]
            if len(f) < 10:
                continue
            try:
                util = float(f[9])
            except ValueError:
                util = 100.0
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9], util))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r, _ in rows for i, v in enumerate(r) if v.lower() == "active"})
        # "under load": samples with the GPU busy (all samples if none is)
        busy = [r for r in rows if r[3] >= 50.0] or rows
        return {"sm_mhz": statistics.median(r[0] for r in busy), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "samples_under_load": len(busy),
                "sm_mhz_all_samples": statistics.median(r[0] for r in rows)}


def rank_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def dist_init(gpus: int):
    rank, local, world = rank_env()
    if world != gpus:
        raise SystemExit(f"bench: --gpus {gpus} but WORLD_SIZE={world}")
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("TRIDI_BENCH_GLOO") != "1" else "gloo")
    return rank, local, world


def free_port() -> int:
    import socket

    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def replica_launch_argv(argv: list[str], gpus: int) -> list[str]:
    """The command that runs this script as `gpus` replica ranks (one process
    per GPU) under torch.distributed.run on this node."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
            "--master-addr=127.0.0.1", f"--master-port={free_port()}", str(Path(__file__).resolve()), *argv]


def barrier(world):
    from tridiagonalsolvers_gb300.distributed import barrier as _barrier

    _barrier()


def max_over_ranks(v: float, world: int, device) -> float:
    from tridiagonalsolvers_gb300.distributed import max_over_ranks as _max

    return _max(v, device)


# ---------------------------------------------------------------------------
# The CPU baselines (cpu_baseline of the GPU arm and the --impl reference arm)
# time the same sample: the first CPU_SAMPLE_M systems of the batch, one
# gold Thomas pass over them per step, on every host core.
CPU_SAMPLE_M = 16384


def cpu_gold_steps(a, b, c, d, threads: int, warmup: int, steps: int):
    """Times `steps` passes of the oracle's gold Thomas (tridiagonal_gold.h:26-53,
    restated in oracle/gold.c) over the sample on `threads` host threads, after
    `warmup` untimed passes; returns (unknowns/s, seconds)."""
    from oracle import gold

    gold.gold_lib()
    for _ in range(max(warmup, 1)):
        gold.serial_many(a, b, c, d, threads=threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        gold.serial_many(a, b, c, d, threads=threads)
    el = time.perf_counter() - t0
    return steps * a.size / el, el


def run_reference(args):
    rank, local, world = rank_env()
    if rank != 0:
        return 0  # replicas: rank 0 alone times the host cores
    from oracle import gold
    from tridiagonalsolvers_gb300 import workloads

    cores = gold.gold_lib().gold_max_threads()
    a, b, c, d = workloads.dominant(CPU_SAMPLE_M, N, seed=workloads.SEEDS["c2"])
    rate, el = cpu_gold_steps(a, b, c, d, cores, args.warmup, args.steps)
    sample_m = CPU_SAMPLE_M
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "unknowns/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_systems_per_step": sample_m, "system_size": N},
        "cpu_baseline": {"value": rate, "unit": "unknowns/s", "cores": cores, "kind": "port",
                         "sample": f"{sample_m} of the {M} systems per step (gold Thomas, FP32, OpenMP over systems), "
                                   f"{args.steps} steps in {el:.2f} s"},
        "e2e": {"value": rate, "unit": "unknowns/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def time_kernel(fn, stream, warmup, iters):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(iters):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / iters


def _per_launch_ms(launch, restore, stream, warmup: int, reps: int) -> float:
    """Median of `reps` single launches timed with CUDA events on `stream`;
    before each, `restore()` copies the inputs afresh (outside the events), so
    every launch sees the same data and the same L2 state.  Each copy is
    queued behind a short device-side delay (~0.2 ms), during which the host
    queues the copy, the events and the launch: the host's launch overhead
    falls before the first event, not between it and the kernel (a launch
    timed on an idle stream measured 11.8 us for a 4.5 us kernel)."""
    import torch

    delay_cycles = 400_000
    pairs = []
    for r in range(warmup + reps):
        torch.cuda._sleep(delay_cycles)  # on the current stream, which is `stream`
        restore()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        launch()
        e1.record(stream)
        if r >= warmup:
            pairs.append((e0, e1))
    stream.synchronize()
    return statistics.median(e0.elapsed_time(e1) for e0, e1 in pairs)


def kernel_table(lib, m: int, n: int, seed: int, dev, peak: float, with_reference: bool, reps: int = 20):
    """This build's FP32 kernels on one seeded batch of m systems x n unknowns
    and, beside each, the reference's own kernel for the same launcher
    rebuilt for sm_103a (its overwrites of a..d undone by a fresh copy before
    every launch; the same copy precedes ours)."""
    import torch

    from tridiagonalsolvers_gb300 import workloads

    a, b, c, d = workloads.dominant(m, n, seed=seed)
    src = [torch.from_numpy(v).to(dev) for v in (a, b, c, d)]
    work = [torch.empty_like(t) for t in src]
    ping = [torch.empty_like(t) for t in src]
    x = torch.empty_like(src[0])
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    wp = [t.data_ptr() for t in (*work, x)]

    def restore():
        for w, t in zip(work, src):
            w.copy_(t)

    ours = {"cr": lambda: lib.tridi_cr_f32(*wp, n, m, sp), "pcr": lambda: lib.tridi_pcr_f32(*wp, n, m, sp),
            "crNBC": lambda: lib.tridi_cr_nbc_f32(*wp, n, m, sp),
            "crNBC32": lambda: lib.tridi_cr_nbc_f32(*wp, n, m, sp)}
    rows = [("cr", "cr", 0), ("pcr", "pcr", 0), ("crNBC", "crNBC", 0), ("crNBC32", "crNBC32", 0)]
    rest = 2
    while rest <= n // 2:
        ours[f"crpcr_rest{rest}"] = (lambda r: lambda: lib.tridi_crpcr_f32(*wp, n, m, r, sp))(rest)
        rows.append((f"crpcr_rest{rest}", "crpcr", rest))
        rest *= 2
    r32 = min(32, n // 2)
    ours[f"crpcrNBC_rest{r32}"] = lambda: lib.tridi_crpcr_nbc_f32(*wp, n, m, r32, sp)
    rows.append((f"crpcrNBC_rest{r32}", "crpcrNBC", r32))
    for g in sorted({8, 64, min(n // 2, 512)}):  # 64: the reference driver's own call (test_tridiagonal.cpp:81)
        ours[f"pcrGauss_g{g}"] = (lambda gg: lambda: lib.tridi_pcr_thomas_f32(*wp, n, m, gg, sp))(g)
        rows.append((f"pcrGauss_g{g}", "pcrGauss", g))
    rk = None
    if with_reference:
        try:
            from oracle.gold import RefKernels

            rk = RefKernels() if RefKernels.available() else None
        except Exception:  # the reference kernels were not built on this machine
            rk = None
    out = {"reference_kernels": "oracle/_ref cubins (reference sources rebuilt for sm_103a)" if rk else
           "not available (reference kernels not built)"}

    def fig(ms):
        gbs = BYTES_PER_UNKNOWN * m * n / (ms * 1e-3) / 1e9
        return {"ms": round(ms, 5), "unknowns_per_s": m * n / (ms * 1e-3), "gbs": round(gbs, 1),
                "frac": round(gbs / peak, 4)}

    for name, kind, param in rows:
        row = {}
        t = _per_launch_ms(lambda: _check_status(ours[name](), name), restore, stream, 3, reps)
        row["ours"] = fig(t)
        if rk is not None:
            try:
                if kind == "pcrGauss":
                    if n > 1024:
                        raise ValueError("the reference's small pcrGauss path takes n <= 1024")
                    launch = lambda: rk.pcr_gauss(*work, *ping, n, m, param, stream.cuda_stream)
                else:
                    launch = lambda: rk.solve(kind, *work, x, n, m, param, stream.cuda_stream)
                tr = _per_launch_ms(launch, restore, stream, 3, reps)
                row["reference"] = fig(tr)
                row["speedup"] = round(tr / t, 3)
            except Exception as e:  # a shape the reference kernel does not launch
                row["reference"] = {"error": str(e)[:100]}
        out[name] = row
    return out


def _check_status(st, what):
    from tridiagonalsolvers_gb300 import _lib

    _lib.check(st, what)


def run_gpu(args):
    import torch

    import tridiagonalsolvers_gb300 as tg
    from tridiagonalsolvers_gb300 import _lib, workloads

    rank, local, world = dist_init(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.lib()
    stream = torch.cuda.current_stream(dev)

    a, b, c, d = workloads.dominant(M, N, seed=workloads.SEEDS["c2"] + rank)
    ta, tb, tc, td = (torch.from_numpy(v).to(dev) for v in (a, b, c, d))
    tx = torch.empty_like(ta)
    sp = ctypes.c_void_p(stream.cuda_stream)
    ptrs = [t.data_ptr() for t in (ta, tb, tc, td, tx)]

    def step():
        _lib.check(lib.tridi_cr_f32(*ptrs, N, M, sp), "tridi_cr_f32")

    # correctness guard on a sample (the timed numbers are meaningless otherwise)
    step()
    torch.cuda.synchronize()
    if rank == 0:
        xs = tx[:32].cpu().numpy()
        res = rel_residual64(a[:32], b[:32], c[:32], d[:32], xs).max()
        if not res < 2e-6:
            raise SystemExit(f"bench: cr result fails the residual check (residual {res:.2e})")

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier(world)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world, dev)
    status = tg.device_status()
    unknowns = M * N
    value = world * unknowns / (ms * 1e-3)

    # ---- end to end through the host-pointer launcher (reference-facing cr()) ----
    ha, hb, hc, hd = (torch.from_numpy(v).pin_memory() for v in (a, b, c, d))
    hx = torch.empty_like(ha).pin_memory()
    hptrs = [t.data_ptr() for t in (ha, hb, hc, hd, hx)]

    def e2e_step():
        _lib.check(lib.tridi_dropin_solve_f32(0, *hptrs, N, M, 0), "tridi_dropin_solve_f32")

    e2e_steps = max(2, min(args.steps, 10))
    for _ in range(2):
        e2e_step()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    barrier(world)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, world, dev)
    if rank == 0:
        res = rel_residual64(a[:32], b[:32], c[:32], d[:32], hx[:32].numpy()).max()
        if not res < 2e-6:
            raise SystemExit(f"bench: drop-in cr result fails the residual check (residual {res:.2e})")
    # the same from ordinary (pageable) host memory, as the reference's own
    # callers allocate it (test_tridiagonal.cpp:34-39); x touched once first
    px = np.ones_like(a)
    pptrs = [v.ctypes.data for v in (a, b, c, d, px)]

    def e2e_pageable_step():
        _lib.check(lib.tridi_dropin_solve_f32(0, *pptrs, N, M, 0), "tridi_dropin_solve_f32")

    e2e_pageable_step()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_pageable_step()
    barrier(world)
    e2e_pg_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, world, dev)
    if rank == 0:
        res = rel_residual64(a[:32], b[:32], c[:32], d[:32], px[:32]).max()
        if not res < 2e-6:
            raise SystemExit(f"bench: pageable drop-in cr result fails the residual check (residual {res:.2e})")

    # ---- per-kernel tables (outside the timed region) ----
    peak, peak_kind = measured_peaks()
    kernels = {}
    tables = {}
    if rank == 0 and not args.no_table:
        cands = [("cr", lambda: lib.tridi_cr_f32(*ptrs, N, M, sp)),
                 ("crNBC", lambda: lib.tridi_cr_nbc_f32(*ptrs, N, M, sp)),
                 ("pcr", lambda: lib.tridi_pcr_f32(*ptrs, N, M, sp)),
                 ("partition", lambda: lib.tridi_solve_f32(*ptrs, N, M, sp)),
                 ("pcrGauss", lambda: lib.tridi_pcr_thomas_f32(*ptrs, N, M, 0, sp))]
        rest = 2
        while rest <= N // 2:
            cands.append((f"crpcr_rest{rest}", (lambda r: lambda: lib.tridi_crpcr_f32(*ptrs, N, M, r, sp))(rest)))
            rest *= 2
        for name, fn in cands:
            t = time_kernel(fn, stream, 3, 20)
            gbs = BYTES_PER_UNKNOWN * unknowns / (t * 1e-3) / 1e9
            kernels[name] = {"ms": round(t, 5), "unknowns_per_s": unknowns / (t * 1e-3), "gbs": round(gbs, 1),
                             "frac": round(gbs / peak, 4)}
        # every plain FP32 shape of the benchmark definitions, each row beside
        # the reference's own kernel rebuilt for sm_103a (a reported baseline)
        with ClockSampler(local) as tclk:
            for (m_, n_, seed_) in ((512, 512, "c1"), (M, N, "c2"), (16384, 1024, "c2b")):
                tables[f"{m_}x{n_}"] = kernel_table(lib, m_, n_, workloads.SEEDS[seed_], dev, peak,
                                                    with_reference=not args.no_reference_kernels)
        tables["clocks"] = tclk.summary()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import gold

        cores = gold.gold_lib().gold_max_threads()
        sm = CPU_SAMPLE_M
        sample = [np.ascontiguousarray(v[:sm]) for v in (a, b, c, d)]
        _, one = cpu_gold_steps(*sample, cores, 3, 1)
        reps = max(20, int(np.ceil(10.0 / max(one, 1e-3))))
        rate, el = cpu_gold_steps(*sample, cores, 0, reps)
        cpu = {"value": rate, "unit": "unknowns/s", "cores": cores, "kind": "port",
               "sample": f"{reps} passes over {sm} of the {M} systems (gold Thomas FP32, {el:.1f} s wall on "
                         f"{cores} threads; the --impl reference arm times the same sample)"}

    if rank == 0:
        achieved = BYTES_PER_UNKNOWN * unknowns / (ms * 1e-3) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": "unknowns/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "num_systems": M, "system_size": N, "solver": "cr",
                       "layout": "contiguous", "l2": "inputs (256 MiB) larger than L2, no flush",
                       "seed": workloads.SEEDS["c2"], "parallelism": f"replicas x{world} (independent batches)"},
            "e2e": {"value": world * unknowns / e2e_s, "unit": "unknowns/s",
                    "h2d_bytes_per_step": 4 * unknowns * 4, "d2h_bytes_per_step": unknowns * 4,
                    "path": "tridi_dropin_solve_f32 (cr() drop-in), pinned host buffers, which the solver "
                            "reads and writes in place over the host link (no staging copies)"},
            "e2e_pageable": {"value": world * unknowns / e2e_pg_s, "unit": "unknowns/s",
                             "h2d_bytes_per_step": 4 * unknowns * 4, "d2h_bytes_per_step": unknowns * 4,
                             "path": "the same drop-in from ordinary (pageable) numpy arrays, " + (
                                 "which the solver reads and writes in place through the host's page tables"
                                 if lib.tridi_dropin_pageable_in_place() else "staged through device memory")},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": profile_traffic(), "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": BYTES_PER_UNKNOWN * unknowns},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": args.steps,
            "device_status": status,
            "kernels": kernels,
            "kernel_tables": tables,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def run_large(args):
    """1024 systems x 65536 unknowns, interleaved, weakly dominant: plain FP32
    large-system solve and FP32 + FP64-residual refinement to 1e-10."""
    import torch

    from tridiagonalsolvers_gb300 import _lib

    lib = _lib.lib()
    dev = torch.device("cuda", 0)
    m, n = 1024, args.large_n
    g = torch.Generator(device=dev)
    g.manual_seed(1003)
    a = torch.rand(n * m, device=dev, generator=g) * 2 - 1
    c = torch.rand(n * m, device=dev, generator=g) * 2 - 1
    a.view(n, m)[0] = 0
    c.view(n, m)[n - 1] = 0
    b = a.abs() + c.abs() + 0.01 + 0.09 * torch.rand(n * m, device=dev, generator=g)
    d = torch.rand(n * m, device=dev, generator=g) * 2 - 1
    x = torch.empty_like(a)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    wsb = lib.tridi_large_workspace_bytes(n, m, 4)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    ptrs = [t.data_ptr() for t in (a, b, c, d, x)]

    def step():
        _lib.check(lib.tridi_solve_large_f32(*ptrs, n, m, 1, ws.data_ptr(), wsb, sp), "tridi_solve_large_f32")

    clk = ClockSampler(0).__enter__()
    ms = time_kernel(step, stream, args.warmup, args.steps)
    x64 = torch.empty(n * m, dtype=torch.float64, device=dev)
    rwsb = lib.tridi_refine_workspace_bytes(n, m, 1)
    rws = torch.empty(rwsb, dtype=torch.uint8, device=dev)
    sweeps, rel = ctypes.c_int(0), ctypes.c_double(0)

    def rstep():
        _lib.check(lib.tridi_refine_f32(*ptrs[:4], x64.data_ptr(), n, m, 1, 1e-10, 20, rws.data_ptr(), rwsb, sp,
                                        ctypes.byref(sweeps), ctypes.byref(rel)), "tridi_refine_f32")

    rms = time_kernel(rstep, stream, 1, max(1, args.steps // 5)) if not args.no_refine else float("nan")
    rstats = (sweeps.value, rel.value)
    rms64 = float("nan")
    if not args.no_refine:  # the same with the native-FP64 residual
        lib.tridi_set_tunable(4, 2)
        rms64 = time_kernel(rstep, stream, 1, max(1, args.steps // 5))
        lib.tridi_set_tunable(4, 0)
    clk.__exit__(None, None, None)
    peak, kind = measured_peaks()
    unknowns = n * m
    line = {
        "metric": METRIC, "value": unknowns / (ms * 1e-3), "unit": "unknowns/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"large-system solve, 1024 systems x {n} unknowns, interleaved, weakly dominant",
                   "seed": 1003, "l2": "inputs (1 GiB) larger than L2"},
        "roofline": {"bound": "hbm", "achieved": BYTES_PER_UNKNOWN * unknowns / (ms * 1e-3) / 1e9, "peak": peak,
                     "unit": "GB/s", "frac": BYTES_PER_UNKNOWN * unknowns / (ms * 1e-3) / 1e9 / peak,
                     "peak_source": kind, "traffic": None},
        "refined": {"value": unknowns / (rms * 1e-3), "ms_per_step": rms, "sweeps": rstats[0],
                    "rel_residual": rstats[1], "tol": 1e-10, "frac_of_plain": ms / rms,
                    "residual_arithmetic": "double-float (FP32 pairs)"},
        "refined_fp64": {"value": unknowns / (rms64 * 1e-3), "ms_per_step": rms64, "sweeps": sweeps.value,
                         "rel_residual": rel.value, "tol": 1e-10, "frac_of_plain": ms / rms64,
                         "residual_arithmetic": "native FP64"},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ragged(args):
    """100000 ADI line systems, sizes log-uniform in [32, 8192]: one persistent
    launch (size-bucketed work queue), plain FP32 and FP32 + FP64-residual
    refinement captured in a CUDA graph."""
    import torch

    from tridiagonalsolvers_gb300 import workloads
    from tridiagonalsolvers_gb300.ragged import RaggedPlan, RaggedRefiner, padded

    dev = torch.device("cuda", 0)
    count = args.ragged_count
    sizes = workloads.ragged_sizes(count, 32, 8192, seed=workloads.SEEDS["c4"])
    a, b, c, d, off = workloads.adi(sizes, seed=workloads.SEEDS["c4"])
    total = int(off[-1])

    def up(v):
        t = torch.zeros(padded(total), dtype=torch.float32, device=dev)
        t[:total] = torch.from_numpy(v)
        return t

    t = [up(v) for v in (a, b, c, d)]
    del a, b, c, d
    # threads per system for each size bucket, timed on this GPU before the plan is built
    from tridiagonalsolvers_gb300 import autotune

    tuned = {}
    if not args.no_autotune:
        for k in autotune.DEFAULT_KEYS["ragged"]:
            if k <= 8192:
                tuned[str(k)] = autotune.tune("ragged", k)[0]
    plan = RaggedPlan(off, device=dev)
    x = torch.zeros(padded(total), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    clk = ClockSampler(0).__enter__()
    ms = time_kernel(lambda: plan.solve(*t, x=x), stream, args.warmup, args.steps)
    clk.__exit__(None, None, None)
    # the refinement's own choice per size bucket (timed on the fused refinement)
    tuned_refine = {}
    if not args.no_autotune:
        for k in autotune.DEFAULT_KEYS["ragged_refine"]:
            if k <= 8192:
                tuned_refine[str(k)] = autotune.tune("ragged_refine", k)[0]
    rplan = RaggedPlan(off, device=dev, refine=True)
    refined = {}
    rclk = ClockSampler(0).__enter__()
    for mode in ("df", "fp64"):
        ref = RaggedRefiner(rplan, *t, sweeps=args.sweeps, graph=True, residual=mode)
        rms = time_kernel(ref.launch, stream, 3, max(3, args.steps // 2))
        _, rel = ref.run()
        refined[mode] = {"value": total / (rms * 1e-3), "ms_per_step": rms, "sweeps": args.sweeps,
                         "rel_residual": rel, "tol": 1e-10, "frac_of_plain": ms / rms, "cuda_graph": True,
                         "residual_arithmetic": {"df": "double-float (FP32 pairs)", "fp64": "native FP64"}[mode]}
        del ref
    rclk.__exit__(None, None, None)
    peak, kind = measured_peaks()
    line = {
        "metric": METRIC, "value": total / (ms * 1e-3), "unit": "unknowns/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"ragged ADI batch, {count} systems, sizes log-uniform in [32, 8192]",
                   "total_unknowns": total, "work_items": plan.items, "seed": workloads.SEEDS["c4"],
                   "l2": "inputs larger than L2",
                   "autotuned_threads_per_system": tuned or "built-in rule (--no-autotune)",
                   "autotuned_threads_per_system_refined": tuned_refine or "built-in rule (--no-autotune)"},
        "roofline": {"bound": "hbm", "achieved": BYTES_PER_UNKNOWN * total / (ms * 1e-3) / 1e9, "peak": peak,
                     "unit": "GB/s", "frac": BYTES_PER_UNKNOWN * total / (ms * 1e-3) / 1e9 / peak,
                     "peak_source": kind,
                     "traffic": (lambda b: b * total if b else None)(
                         profile_value("ragged_100000_ncu.md", "traffic_bytes_per_row")),
                     "traffic_note": "ncu dram bytes per row of a 20000-system capture, scaled to this batch"},
        "refined": refined["df"],
        "refined_fp64": refined["fp64"],
        "clocks": clk.summary(),
        "clocks_refined": rclk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_serve(args):
    """Served request stream: requests of 1..4096 systems of 64..16384 unknowns
    (log-uniform; diagonally dominant or ADI), host arrays in, FP64 x out,
    refined to 1e-10 by the continuous-batching server.  First all requests
    at once (saturation throughput), then Poisson arrivals at fractions of
    that rate (p50 / p99 latency).  The plain FP32 form of the same rows on
    the same GPU is timed beside it: device-resident (one ragged launch) and
    end to end (pinned host buffers in and out)."""
    import threading

    import torch

    from tridiagonalsolvers_gb300.ragged import RaggedPlan, padded
    from tridiagonalsolvers_gb300.serve import Server, make_request

    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(workloads_seed("c5"))
    pool = [make_request(rng) for _ in range(args.serve_requests)]
    rows = [int(r[4][-1]) for r in pool]
    total = sum(rows)
    from tridiagonalsolvers_gb300 import _lib

    L = _lib.lib()
    copy_mode = {"auto": 0, "memcpy": 1, "direct": 2, "staged": 3}[args.server_copy]
    L.tridi_set_tunable(5, copy_mode)  # TRIDI_TUNE_SERVER_COPY, read when the server is created
    srv = Server(hbm_budget_bytes=48 << 30, max_batch_rows=1 << 24, max_inflight=args.server_slots,
                 sweeps=args.sweeps, max_sweeps=args.sweeps + 2)

    # one output buffer per request, allocated and touched once (a serving
    # loop reuses its result buffers; first-touch page faults stay out of the timing)
    outs = [np.zeros(r, dtype=np.float64) for r in rows]
    for o in outs:
        o.fill(1.0)

    def serve_once(arrivals):
        """Submits pool[i] at arrivals[i] seconds after the start; returns
        (wall seconds, per-request info)."""
        ids = [None] * len(pool)
        t0 = time.perf_counter()
        for i, (a, b, c, d, off) in enumerate(pool):
            delay = arrivals[i] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            ids[i] = srv.submit(a, b, c, d, off, tol=1e-10, out=outs[i])
        infos = [srv.wait(rid)[1] for rid in ids]
        return time.perf_counter() - t0, infos

    # warm up: one untimed pass of the whole stream at saturation (kernels
    # loaded, the server's memory pool grown to its steady size, host pages
    # of the request and result arrays touched), as a serving loop that has
    # been running would be
    serve_once([0.0] * len(pool))
    clk = ClockSampler(0).__enter__()
    wall, infos = serve_once([0.0] * len(pool))
    sat = total / wall
    def lat(infos):
        v = np.array([i["latency_us"] for i in infos]) / 1e3
        return {"p50_ms": float(np.percentile(v, 50)), "p99_ms": float(np.percentile(v, 99)),
                "max_rel_residual": max(i["rel_residual"] for i in infos),
                "sweeps_max": max(i["sweeps"] for i in infos)}
    sweep = [{"offered_frac_of_saturation": 1.0, "arrivals": "all at t=0", "unknowns_per_s": sat, **lat(infos)}]
    req_rate = len(pool) / wall
    arng = np.random.default_rng(workloads_seed("c5") + 1)
    for frac in (0.5, 0.8):
        gaps = arng.exponential(1.0 / (frac * req_rate), len(pool))
        arr = np.concatenate([[0.0], np.cumsum(gaps[:-1])])
        w, inf = serve_once(arr)
        sweep.append({"offered_frac_of_saturation": frac, "arrivals": "poisson", "rate_req_per_s": frac * req_rate,
                      "unknowns_per_s": total / w, **lat(inf)})
    stats = srv.stats()
    stats["worker_phase_ms"] = srv.phase_ms()
    srv.close()

    # plain FP32 form of the same rows on the same GPU
    off_all = np.concatenate([[0], np.cumsum(rows)]).astype(np.int64)
    sys_off = [0]
    for r in pool:
        o = r[4]
        sys_off.extend((o[1:] + sys_off[-1]).tolist())
    sys_off = np.array(sys_off, dtype=np.int64)
    cat = [np.concatenate([r[q] for r in pool]) for q in range(4)]
    need = padded(total)
    host = []
    for v in cat:
        h = torch.zeros(need, dtype=torch.float32).pin_memory()
        h[:total] = torch.from_numpy(v)
        host.append(h)
    hx = torch.zeros(need, dtype=torch.float32).pin_memory()
    dv = [torch.empty(need, dtype=torch.float32, device=dev) for _ in range(4)]
    dx = torch.empty(need, dtype=torch.float32, device=dev)
    for h, t in zip(host, dv):
        t.copy_(h)
    plan = RaggedPlan(sys_off, device=dev)
    stream = torch.cuda.current_stream(dev)
    ms_dev = time_kernel(lambda: plan.solve(*dv, x=dx), stream, 3, 10)

    def e2e():
        for h, t in zip(host, dv):
            t.copy_(h, non_blocking=True)
        plan.solve(*dv, x=dx)
        hx.copy_(dx, non_blocking=True)
        torch.cuda.synchronize()

    e2e()
    t0 = time.perf_counter()
    for _ in range(5):
        e2e()
    e2e_s = (time.perf_counter() - t0) / 5
    # the same from the pageable host arrays the server is given (x into a touched float32 array)
    pg_in = [torch.from_numpy(np.ascontiguousarray(v)) for v in cat]
    pg_out = torch.ones(total, dtype=torch.float32)

    def e2e_pageable():
        for h, t in zip(pg_in, dv):
            t[:total].copy_(h)
        plan.solve(*dv, x=dx)
        pg_out.copy_(dx[:total])

    e2e_pageable()
    t0 = time.perf_counter()
    for _ in range(5):
        e2e_pageable()
    e2e_pg_s = (time.perf_counter() - t0) / 5
    clk.__exit__(None, None, None)
    plain_dev = total / (ms_dev * 1e-3)
    plain_e2e = total / e2e_s
    plain_e2e_pg = total / e2e_pg_s
    del off_all
    line = {
        "metric": METRIC, "value": sat, "unit": "unknowns/s", "n_gpus": 1, "steps": len(pool), "warmup": len(pool),
        "ms_per_step": wall / len(pool) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 solves, double-float residual, f64 x", "data": "synthetic",
        "config": {"workload": f"served request stream, {len(pool)} requests of 1-4096 systems x 64-16384 unknowns "
                               "(log-uniform, dominant or ADI), refined to 1e-10",
                   "total_unknowns": total, "seed": workloads_seed("c5"), "sweeps": args.sweeps,
                   "server": {"hbm_budget_gb": 48, "max_batch_rows": 1 << 24, "max_inflight": args.server_slots,
                              "host_transfer": args.server_copy}},
        "e2e": {"value": sat, "unit": "unknowns/s", "h2d_bytes_per_step": 16 * total / len(pool),
                "d2h_bytes_per_step": 8 * total / len(pool), "path": "tridi_server_submit / tridi_server_wait"},
        "latency_sweep": sweep,
        "server_stats": stats,
        "plain_fp32_same_rows": {"device_resident_unknowns_per_s": plain_dev,
                                 "e2e_pinned_unknowns_per_s": plain_e2e,
                                 "e2e_pageable_unknowns_per_s": plain_e2e_pg,
                                 "served_frac_of_plain_e2e_pinned": sat / plain_e2e,
                                 "served_frac_of_plain_e2e_pageable": sat / plain_e2e_pg,
                                 "served_frac_of_plain_device": sat / plain_dev},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


KERNELS = ("cr", "pcr", "crpcr", "crNBC", "crNBC32", "crpcrNBC", "pcrGauss", "partition", "large", "refine")


def run_kernel(args):
    """One solver of the family on one seeded batch (`--kernel`, `--system-size`,
    `--num-systems`, `--param` = rest / gaussian, `--tunable KEY=VALUE`):
    W untimed and K timed launches back to back on one stream, CUDA events.
    Strictly diagonally dominant inputs (weakly dominant and interleaved for
    large / refine).  Also the command that ncu captures of one kernel run."""
    import torch

    from tridiagonalsolvers_gb300 import _lib, solvers, workloads

    lib = _lib.lib()
    for kv in args.tunable:
        key, val = (int(v) for v in kv.split("="))
        _lib.check(lib.tridi_set_tunable(key, val), "tridi_set_tunable")
    dev = torch.device("cuda", 0)
    n, m, kind = args.system_size, args.num_systems, args.kernel
    inter = kind in ("large", "refine")
    gen = workloads.weak if inter else workloads.dominant
    a, b, c, d = gen(m, n, seed=workloads.SEEDS["c2"], layout=1 if inter else 0)
    t = [torch.from_numpy(v).to(dev).reshape(-1) for v in (a, b, c, d)]
    x = torch.empty_like(t[0])
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    ptrs = [v.data_ptr() for v in (*t, x)]
    param = args.param
    direct = {
        "cr": lambda: lib.tridi_cr_f32(*ptrs, n, m, sp), "pcr": lambda: lib.tridi_pcr_f32(*ptrs, n, m, sp),
        "crpcr": lambda: lib.tridi_crpcr_f32(*ptrs, n, m, param or 32, sp),
        "crNBC": lambda: lib.tridi_cr_nbc_f32(*ptrs, n, m, sp), "crNBC32": lambda: lib.tridi_cr_nbc_f32(*ptrs, n, m, sp),
        "crpcrNBC": lambda: lib.tridi_crpcr_nbc_f32(*ptrs, n, m, param or 32, sp),
        "pcrGauss": lambda: lib.tridi_pcr_thomas_f32(*ptrs, n, m, param, sp),
        "partition": lambda: lib.tridi_solve_f32(*ptrs, n, m, sp),
    }
    if kind in direct:
        def step():
            _lib.check(direct[kind](), kind)
    elif kind == "large":
        wsb = lib.tridi_large_workspace_bytes(n, m, 4)
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)

        def step():
            _lib.check(lib.tridi_solve_large_f32(*ptrs, n, m, 1, ws.data_ptr(), wsb, sp), "tridi_solve_large_f32")
    else:
        x64 = torch.empty(n * m, dtype=torch.float64, device=dev)

        def step():
            solvers.refine(*t, n, m, layout="interleaved", tol=1e-10, max_sweeps=20, x=x64)
    with ClockSampler(0) as clk:
        ms = time_kernel(step, stream, args.warmup, args.steps)
    peak, peak_kind = measured_peaks()
    bpu = 24 if kind == "refine" else BYTES_PER_UNKNOWN
    gbs = bpu * n * m / (ms * 1e-3) / 1e9
    line = {"metric": METRIC, "value": n * m / (ms * 1e-3), "unit": "unknowns/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{kind}, {m} systems x {n} unknowns" + (", interleaved" if inter else ""),
                       "param": param, "tunables": args.tunable, "seed": workloads.SEEDS["c2"],
                       "l2": "back-to-back launches"},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "peak_source": peak_kind, "bytes_per_unknown": bpu},
            "clocks": clk.summary(), "device_status": solvers.device_status()}
    print(json.dumps(line), flush=True)
    return 0


def workloads_seed(tag):
    from tridiagonalsolvers_gb300 import workloads

    return workloads.SEEDS[tag]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-table", action="store_true", help="skip the per-kernel table")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-reference-kernels", action="store_true",
                    help="per-kernel tables without the reference's own kernels beside them")
    ap.add_argument("--workload", default="batch", choices=["batch", "large", "ragged", "serve", "kernel"],
                    help="batch: 65536 x 256 (default, the headline); large: 1024 x 65536 interleaved; "
                         "ragged: 100000 ADI systems of 32..8192 unknowns; serve: a served request stream; "
                         "kernel: one solver (--kernel) on one batch")
    ap.add_argument("--kernel", default="cr", choices=KERNELS, help="kernel workload: the solver")
    ap.add_argument("--system-size", type=int, default=N, help="kernel workload: unknowns per system")
    ap.add_argument("--num-systems", type=int, default=M, help="kernel workload: systems")
    ap.add_argument("--param", type=int, default=0, help="kernel workload: rest (crpcr) or gaussian (pcrGauss)")
    ap.add_argument("--tunable", action="append", default=[], metavar="KEY=VALUE",
                    help="kernel workload: tridi_set_tunable before the run (repeatable)")
    ap.add_argument("--ragged-count", type=int, default=100000, help="systems of the ragged workload")
    ap.add_argument("--sweeps", type=int, default=1, help="refinement sweeps of the ragged / serve workloads")
    ap.add_argument("--serve-requests", type=int, default=200, help="requests of the serve workload")
    ap.add_argument("--no-autotune", action="store_true", help="ragged workload: keep the built-in size classes")
    ap.add_argument("--server-copy", default="auto", choices=["auto", "memcpy", "direct", "staged"],
                    help="serve workload: host transfer (auto = the server's default, cudaMemcpyAsync on the "
                         "callers' arrays; staged = through pinned buffers filled by host threads; "
                         "direct = the GPU reads / writes the callers' arrays)")
    ap.add_argument("--server-slots", type=int, default=4, help="serve workload: concurrent batches")
    ap.add_argument("--large-n", type=int, default=65536, help="system size of the large workload")
    ap.add_argument("--no-refine", action="store_true", help="large workload: plain solve only")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # N independent replicas, one process per GPU
        argv = replica_launch_argv(sys.argv[1:], args.gpus)
        return subprocess.run(argv).returncode
    if args.warmup < 3 and args.impl == "native":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "large":
        return run_large(args)
    if args.workload == "ragged":
        return run_ragged(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "kernel":
        return run_kernel(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
