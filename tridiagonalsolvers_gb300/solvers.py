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


def device_status(reset: bool = True) -> int:
    """Synchronises and returns the TRIDI_DEVERR_* bits of the current device."""
    bits = ctypes.c_uint(0)
    check(lib().tridi_device_status(ctypes.byref(bits), int(reset)), "tridi_device_status")
    return bits.value
