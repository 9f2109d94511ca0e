"""Ragged batches on the GPU: systems of different sizes in one persistent
launch (tridi_ragged_* of include/tridi.h).

    plan = RaggedPlan(offsets)          # host int64 array, num_systems + 1 entries
    x = plan.solve(a, b, c, d)          # flat float32 CUDA tensors, concatenated rows

The plan (size buckets, work items) is built once and reused; `padded(n)`
gives the allocation length the arrays need (a multiple of 4 elements).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib


def padded(total_rows: int) -> int:
    return (int(total_rows) + 3) & ~3


class RaggedPlan:
    """refine=True: a plan for RaggedRefiner, with threads per system from the
    refinement's tuning table ("ragged_refine") where it was tuned."""

    def __init__(self, offsets, device=None, refine: bool = False):
        import torch

        off = np.ascontiguousarray(np.asarray(offsets, dtype=np.int64))
        if off.ndim != 1 or len(off) < 2 or off[0] != 0 or np.any(np.diff(off) <= 0):
            raise ValueError("offsets must start at 0 and increase strictly")
        self.offsets = off
        self.num_systems = len(off) - 1
        self.total_rows = int(off[-1])
        L = lib()
        h = ctypes.c_void_p()
        create = L.tridi_ragged_plan_create_refine if refine else L.tridi_ragged_plan_create
        check(create(off.ctypes.data, self.num_systems, ctypes.byref(h)), "ragged plan")
        self._h = h
        self.items = L.tridi_ragged_plan_items(h)
        nbytes = L.tridi_ragged_plan_device_bytes(h)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._dev = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        check(L.tridi_ragged_plan_upload(h, self._dev.data_ptr(), nbytes, stream), "ragged plan upload")

    def solve(self, a, b, c, d, x=None):
        import torch

        need = padded(self.total_rows)
        for t in (a, b, c, d):
            if t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous() or t.numel() < need:
                raise ValueError(f"a, b, c, d must be contiguous float32 CUDA tensors of >= {need} elements")
        if x is None:
            x = torch.zeros(need, dtype=torch.float32, device=a.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
        check(lib().tridi_ragged_solve_f32(a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(), x.data_ptr(),
                                           self._h, self._dev.data_ptr(), stream), "tridi_ragged_solve_f32")
        return x

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().tridi_ragged_plan_destroy(h)
            except Exception:
                pass
            self._h = None


TUNE_RESIDUAL = 4  # TRIDI_TUNE_RESIDUAL
RESIDUAL_MODES = {"df": 1, "fp64": 2}  # TRIDI_RESIDUAL_DF, TRIDI_RESIDUAL_FP64


class RaggedRefiner:
    """Fused mixed-precision refinement of a ragged batch (one launch): FP32
    solves, residual and update in extended precision -- "df" (double-float,
    pairs of FP32) or "fp64" (native) -- a fixed number of correction sweeps,
    optionally captured once in a CUDA graph and replayed.

        r = RaggedRefiner(plan, a, b, c, d, sweeps=1, graph=True)
        x64, rel = r.run()       # FP64 solution (padded rows) and max relative residual
    """

    def __init__(self, plan: RaggedPlan, a, b, c, d, sweeps: int = 1, graph: bool = True, residual: str = "df"):
        import torch

        L = lib()
        check(L.tridi_init(), "tridi_init")  # status word allocated outside any capture
        if residual not in RESIDUAL_MODES:
            raise ValueError(f"residual must be one of {sorted(RESIDUAL_MODES)}")
        self.residual = residual
        self.plan, self.sweeps = plan, int(sweeps)
        self.inputs = (a, b, c, d)
        dev = a.device
        need = padded(plan.total_rows)
        self.x = torch.zeros(need, dtype=torch.float64, device=dev)
        self.rel = torch.zeros(1, dtype=torch.float64, device=dev)
        self.off = torch.from_numpy(plan.offsets).to(dev)
        wsb = L.tridi_ragged_refine_workspace_bytes(plan.total_rows, plan.num_systems)
        self.ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        self._wsb = wsb
        self.graph = None
        if graph:
            self._launch()  # warm up: kernel attributes set, everything resident
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="relaxed"):
                self._launch()
            self.graph = g

    def _launch(self):
        import torch

        a, b, c, d = self.inputs
        L = lib()
        stream = ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
        prev = L.tridi_get_tunable(TUNE_RESIDUAL)
        check(L.tridi_set_tunable(TUNE_RESIDUAL, RESIDUAL_MODES[self.residual]), "tridi_set_tunable")
        try:
            check(L.tridi_ragged_refine_f32(a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(),
                                            self.x.data_ptr(), self.plan._h, self.plan._dev.data_ptr(),
                                            self.off.data_ptr(), self.sweeps, self.ws.data_ptr(), self._wsb,
                                            self.rel.data_ptr(), stream), "tridi_ragged_refine_f32")
        finally:
            L.tridi_set_tunable(TUNE_RESIDUAL, prev)

    def launch(self):
        """Enqueue one refined solve (graph replay if captured); no sync."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._launch()

    def run(self):
        import torch

        self.launch()
        torch.cuda.synchronize()
        return self.x, float(self.rel.item())
