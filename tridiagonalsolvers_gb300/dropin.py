"""The reference's host launchers on numpy arrays (host memory), through the
C ABI's host-pointer entry points (tridi_dropin_solve_f32 / _f64).

    cr(a, b, c, d, x, system_size, num_systems)
    pcr(...), crNBC(...), crNBC32(...)
    crpcr(a, b, c, d, x, system_size, num_systems, rest_system_size)
    crpcrNBC(...same...)
    pcrGaussWrapper(a, b, c, d, x, system_size, num_systems, gaussian)

Same argument order and meaning as cr_app.cu:4, pcr_app.cu:5, crpcr_app.cu:5,
crNBC.cu:123/344, crNBC32banks.cu:123, pcrGauss_app.cu:164: host arrays in
the contiguous layout, x receives the solution, a..d are left unchanged, the
call is synchronous.  Errors raise TridiError (the C++ drop-ins print and exit
like the reference's CUDA_SAFE_CALL; a Python caller gets an exception).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, lib

CR, PCR, CRPCR, CR_NBC, CRPCR_NBC, CR_NBC32, PCR_THOMAS = range(7)


def _solve(algo, a, b, c, d, x, system_size, num_systems, param=0):
    arrs = [a, b, c, d, x]
    dt = np.asarray(a).dtype
    if dt not in (np.float32, np.float64):
        raise TypeError(f"unsupported dtype {dt}")
    for v in arrs:
        if not isinstance(v, np.ndarray) or v.dtype != dt or not v.flags.c_contiguous:
            raise ValueError("a, b, c, d, x must be C-contiguous numpy arrays of one float dtype")
        if v.size < system_size * num_systems:
            raise ValueError("array smaller than system_size * num_systems")
    if not x.flags.writeable:
        raise ValueError("x must be writeable")
    suf = "f32" if dt == np.float32 else "f64"
    fn = getattr(lib(), f"tridi_dropin_solve_{suf}")
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 5 + [ctypes.c_int] * 3
    check(fn(algo, *(v.ctypes.data for v in arrs), int(system_size), int(num_systems), int(param)),
          f"drop-in algo {algo} (n={system_size}, m={num_systems})")
    return x


def cr(a, b, c, d, x, system_size, num_systems):
    return _solve(CR, a, b, c, d, x, system_size, num_systems)


def pcr(a, b, c, d, x, system_size, num_systems):
    return _solve(PCR, a, b, c, d, x, system_size, num_systems)


def crpcr(a, b, c, d, x, system_size, num_systems, rest_system_size):
    return _solve(CRPCR, a, b, c, d, x, system_size, num_systems, rest_system_size)


def crNBC(a, b, c, d, x, system_size, num_systems):
    return _solve(CR_NBC, a, b, c, d, x, system_size, num_systems)


def crpcrNBC(a, b, c, d, x, system_size, num_systems, rest_system_size):
    return _solve(CRPCR_NBC, a, b, c, d, x, system_size, num_systems, rest_system_size)


def crNBC32(a, b, c, d, x, system_size, num_systems):
    return _solve(CR_NBC32, a, b, c, d, x, system_size, num_systems)


def pcrGaussWrapper(a, b, c, d, x, system_size, num_systems, gaussian):
    return _solve(PCR_THOMAS, a, b, c, d, x, system_size, num_systems, gaussian)


def write_result_file(x, num_systems, system_size, path):
    """The reference driver's text dump of a solution (writeResultToFile,
    tridiagonal_gold.h:96-107): per system a header line, then one value per
    line, C++ default stream format.  x: host float32 or float64 array."""
    x = np.ascontiguousarray(x)
    if x.size < num_systems * system_size:
        raise ValueError("x shorter than num_systems * system_size")
    fn = {np.dtype(np.float32): "tridi_write_result_file_f32",
          np.dtype(np.float64): "tridi_write_result_file_f64"}.get(x.dtype)
    if fn is None:
        raise TypeError("x must be float32 or float64")
    check(getattr(lib(), fn)(x.ctypes.data, int(num_systems), int(system_size), str(path).encode()), fn)
