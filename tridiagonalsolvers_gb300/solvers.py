"""Device-tensor front end of the C ABI (include/tridi.h).

The functions keep the reference launchers' names and argument meaning
(a, b, c, d, x, system_size, num_systems[, rest_system_size]); the
difference is that a..d and x are device tensors (the host-pointer,
allocate-copy-solve-copy form of the reference lives in the C++ drop-in
library, include/tridi_dropin.h, and in tridiagonalsolvers_gb300.dropin).
Inputs are never modified.
"""
from __future__ import annotations

import ctypes

from ._lib import check, lib


def _torch():
    import torch

    return torch


def _prep(a, b, c, d, x, system_size):
    torch = _torch()
    ts = (a, b, c, d)
    dt = a.dtype
    if dt not in (torch.float32, torch.float64):
        raise TypeError(f"unsupported dtype {dt}")
    for t in ts:
        if not t.is_cuda:
            raise ValueError("inputs must be CUDA tensors")
        if t.dtype != dt or t.numel() != a.numel():
            raise ValueError("a, b, c, d must share dtype and size")
        if not t.is_contiguous():
            raise ValueError("inputs must be contiguous")
    n = int(system_size if system_size is not None else a.shape[-1])
    if n <= 0 or a.numel() % n:
        raise ValueError(f"numel {a.numel()} is not a multiple of system_size {n}")
    m = a.numel() // n
    if x is None:
        x = torch.empty_like(a)
    elif x.dtype != dt or x.numel() != a.numel() or not x.is_cuda or not x.is_contiguous():
        raise ValueError("x must be a contiguous CUDA tensor like a")
    suf = "f32" if dt == torch.float32 else "f64"
    stream = ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
    return ts, x, n, m, suf, stream


def _call(name, a, b, c, d, x, system_size, *extra):
    ts, x, n, m, suf, stream = _prep(a, b, c, d, x, system_size)
    fn = getattr(lib(), f"tridi_{name}_{suf}")
    ptrs = [t.data_ptr() for t in ts]
    check(fn(*ptrs, x.data_ptr(), n, m, *extra, stream), f"tridi_{name}_{suf}(n={n}, m={m})")
    return x


def cr(a, b, c, d, x=None, system_size=None):
    """Cyclic reduction (cr_app.cu:4 / cr_kernel.cu)."""
    return _call("cr", a, b, c, d, x, system_size)


def pcr(a, b, c, d, x=None, system_size=None):
    """Parallel cyclic reduction (pcr_app.cu:5 / pcr_kernel.cu)."""
    return _call("pcr", a, b, c, d, x, system_size)


def crpcr(a, b, c, d, rest_system_size, x=None, system_size=None):
    """Hybrid CR -> PCR -> CR; rest_system_size is the intermediate system's size
    (crpcr_app.cu:5 / crpcr_kernel.cu)."""
    return _call("crpcr", a, b, c, d, x, system_size, int(rest_system_size))


def crNBC(a, b, c, d, x=None, system_size=None):
    """Bank-conflict-free shared-memory CR (crNBC.cu:123)."""
    return _call("cr_nbc", a, b, c, d, x, system_size)


def crNBC32(a, b, c, d, x=None, system_size=None):
    """crNBC32banks.cu:123; the same bank-conflict-free CR as crNBC."""
    return _call("cr_nbc", a, b, c, d, x, system_size)


def crpcrNBC(a, b, c, d, rest_system_size, x=None, system_size=None):
    """Hybrid with the bank-conflict-free CR part (crNBC.cu:344)."""
    return _call("crpcr_nbc", a, b, c, d, x, system_size, int(rest_system_size))


def pcrGauss(a, b, c, d, gaussian, x=None, system_size=None):
    """PCR-then-Thomas with `gaussian` interleaved subsystems (pcrGauss_app.cu:164),
    exact for every power-of-two gaussian; gaussian = 0 takes the autotuned
    split for this size (else n/2 for power-of-two n: log2(n/2) PCR steps and
    2-row chains, solved by the register PCR kernels)."""
    return _call("pcr_thomas", a, b, c, d, x, system_size, int(gaussian))


def solve(a, b, c, d, x=None, system_size=None):
    """Generic batched solve of any size (partition method, tridi_solve_*)."""
    return _call("solve", a, b, c, d, x, system_size)


def solve_large(a, b, c, d, system_size, num_systems, layout="contiguous", x=None):
    """Large systems in either layout (tridi_solve_large_*): flat CUDA tensors,
    layout "contiguous" (s*n + i) or "interleaved" (i*num_systems + s)."""
    torch = _torch()
    lay = {"contiguous": 0, "interleaved": 1}[layout]
    n, m = int(system_size), int(num_systems)
    ts = (a, b, c, d)
    for t in ts:
        if not t.is_cuda or t.numel() != n * m or not t.is_contiguous() or t.dtype != a.dtype:
            raise ValueError("a, b, c, d must be contiguous CUDA tensors of n*m elements")
    if x is None:
        x = torch.empty_like(a)
    suf = "f32" if a.dtype == torch.float32 else "f64"
    L = lib()
    ws_bytes = L.tridi_large_workspace_bytes(n, m, a.element_size())
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=a.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
    fn = getattr(L, f"tridi_solve_large_{suf}")
    check(fn(*(t.data_ptr() for t in ts), x.data_ptr(), n, m, lay, ws.data_ptr(), ws_bytes, stream),
          f"tridi_solve_large_{suf}(n={n}, m={m}, {layout})")
    return x


def refine(a, b, c, d, system_size, num_systems, layout="contiguous", tol=1e-10, max_sweeps=10, x=None,
           residual="df"):
    """FP32 solves + extended-precision residual refinement (tridi_refine_f32):
    residual and update in double-float ("df", FP32 pairs) or native FP64
    ("fp64").  a..d float32 CUDA tensors (flat, n*m), returns (x float64,
    sweeps, max relative residual).  Raises TridiError if the tolerance is not
    met within max_sweeps."""
    torch = _torch()
    lay = {"contiguous": 0, "interleaved": 1}[layout]
    n, m = int(system_size), int(num_systems)
    for t in (a, b, c, d):
        if t.dtype != torch.float32 or not t.is_cuda or t.numel() != n * m or not t.is_contiguous():
            raise ValueError("a, b, c, d must be contiguous float32 CUDA tensors of n*m elements")
    if x is None:
        x = torch.empty(n * m, dtype=torch.float64, device=a.device)
    L = lib()
    wsb = L.tridi_refine_workspace_bytes(n, m, lay)
    ws = torch.empty(wsb, dtype=torch.uint8, device=a.device)
    sweeps = ctypes.c_int(0)
    rel = ctypes.c_double(0.0)
    stream = ctypes.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)
    mode = {"df": 1, "fp64": 2}[residual]  # TRIDI_RESIDUAL_DF / TRIDI_RESIDUAL_FP64
    prev = L.tridi_get_tunable(4)  # TRIDI_TUNE_RESIDUAL
    check(L.tridi_set_tunable(4, mode), "tridi_set_tunable")
    try:
        check(L.tridi_refine_f32(a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(), x.data_ptr(), n, m, lay,
                                 float(tol), int(max_sweeps), ws.data_ptr(), wsb, stream, ctypes.byref(sweeps),
                                 ctypes.byref(rel)), f"tridi_refine_f32(n={n}, m={m}, {layout})")
    finally:
        L.tridi_set_tunable(4, prev)
    return x, sweeps.value, rel.value


def device_status(reset: bool = True) -> int:
    """Synchronises and returns the TRIDI_DEVERR_* bits of the current device."""
    bits = ctypes.c_uint(0)
    check(lib().tridi_device_status(ctypes.byref(bits), int(reset)), "tridi_device_status")
    return bits.value
