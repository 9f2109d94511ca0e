"""Python face of the continuous-batching solve server (tridi_server_* of
include/tridi.h; the scheduler, admission and batching are C++ in the library).

    srv = Server(hbm_budget_bytes=8 << 30)
    rid = srv.submit(a, b, c, d, offsets)     # host float32 arrays, int64 offsets
    x, info = srv.wait(rid)                   # float64 solution, status/sweeps/residual/latency
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import TridiError, check, lib


class Server:
    def __init__(self, hbm_budget_bytes: int = 8 << 30, max_batch_rows: int = 1 << 24, max_inflight: int = 3,
                 sweeps: int = 1, max_sweeps: int = 4):
        self._h = ctypes.c_void_p()
        check(lib().tridi_server_create(int(hbm_budget_bytes), int(max_batch_rows), int(max_inflight), int(sweeps),
                                        int(max_sweeps), ctypes.byref(self._h)), "tridi_server_create")
        self._live = {}  # id -> arrays kept alive until wait

    @staticmethod
    def footprint(rows: int, num_systems: int) -> int:
        return int(lib().tridi_server_request_footprint(int(rows), int(num_systems)))

    def submit(self, a, b, c, d, offsets, tol: float = 1e-10, out=None) -> int:
        """Queues one request; `out` (float64, >= offsets[-1] elements, e.g. a
        reused buffer) receives x, else a new array does."""
        arrs = [np.ascontiguousarray(v, dtype=np.float32) for v in (a, b, c, d)]
        off = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        rows = int(off[-1])
        if any(v.size < rows for v in arrs):
            raise ValueError("arrays shorter than offsets[-1]")
        if out is None:
            x = np.empty(rows, dtype=np.float64)
        else:
            if out.dtype != np.float64 or not out.flags.c_contiguous or out.size < rows:
                raise ValueError("out must be a contiguous float64 array of >= offsets[-1] elements")
            x = out
        rid = ctypes.c_longlong(0)
        check(lib().tridi_server_submit(self._h, *(v.ctypes.data for v in arrs), x.ctypes.data, off.ctypes.data,
                                        len(off) - 1, float(tol), ctypes.byref(rid)), "tridi_server_submit")
        self._live[rid.value] = (arrs, off, x)
        return rid.value

    def wait(self, rid: int, timeout_ms: int = -1):
        st, sw = ctypes.c_int(0), ctypes.c_int(0)
        rel, lat = ctypes.c_double(0), ctypes.c_double(0)
        check(lib().tridi_server_wait(self._h, rid, int(timeout_ms), ctypes.byref(st), ctypes.byref(sw),
                                      ctypes.byref(rel), ctypes.byref(lat)), f"wait({rid})")
        _, _, x = self._live.pop(rid)
        info = {"status": st.value, "sweeps": sw.value, "rel_residual": rel.value, "latency_us": lat.value}
        if st.value != 0:
            raise TridiError(st.value, f"request {rid}")
        return x, info

    def stats(self):
        c, b, r = ctypes.c_longlong(0), ctypes.c_longlong(0), ctypes.c_longlong(0)
        mi = ctypes.c_double(0)
        check(lib().tridi_server_stats(self._h, ctypes.byref(c), ctypes.byref(b), ctypes.byref(r), ctypes.byref(mi)),
              "stats")
        return {"completed": c.value, "batches": b.value, "rows": r.value, "max_inflight_seen": mi.value}

    def phase_ms(self):
        """Milliseconds the slot workers spent per phase, summed over batches."""
        v = (ctypes.c_double * 5)()
        check(lib().tridi_server_phase_times(self._h, v, 5), "phase times")
        names = ("plan", "alloc_h2d", "refine", "d2h", "release")
        return {k: v[i] / 1e3 for i, k in enumerate(names)}

    def close(self):
        if self._h and self._h.value:
            lib().tridi_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_request(rng, max_systems=4096, lo=64, hi=16384, kind=None):
    """One request of the served workload: 1..max_systems systems (log-uniform)
    of lo..hi unknowns (log-uniform), from the dominant or the ADI family."""
    from . import workloads

    k = int(np.exp(rng.uniform(0, np.log(max_systems + 1))))
    k = max(1, min(max_systems, k))
    sizes = np.clip(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), k)).astype(np.int64), lo, hi)
    seed = int(rng.integers(1 << 31))
    kind = kind or ("adi" if rng.random() < 0.5 else "dominant")
    if kind == "adi":
        a, b, c, d, off = workloads.adi(sizes, seed=seed)
    else:
        g = np.random.default_rng(seed)
        off = np.zeros(k + 1, np.int64)
        np.cumsum(sizes, out=off[1:])
        n = int(off[-1])
        a = g.uniform(-1, 1, n)
        c = g.uniform(-1, 1, n)
        a[off[:-1]] = 0
        c[off[1:] - 1] = 0
        b = np.abs(a) + np.abs(c) + g.uniform(1, 2, n)
        d = g.uniform(-1, 1, n)
        a, b, c, d = (v.astype(np.float32) for v in (a, b, c, d))
    return a, b, c, d, off
