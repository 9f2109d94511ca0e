"""Python face of the oracle (test infrastructure only).

The CPU restatement of the reference's gold solver (oracle/gold.c, built into
oracle/_build/libgold.so), the reference's own gold routines where they were
compiled here (oracle/_ref/libgold_ref_*.so), and the launcher of the
reference's own GPU kernels (oracle/ref_kernels_runner.cpp over the cubins in
oracle/_ref/{f32,f64}/).  Only the tests, the smoke check and bench.py's
CPU-baseline leg import this module; the product never does.
"""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_uint, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF = HERE / "_ref"

_gold = None
_ref = {}
_runner = None

F32P = POINTER(c_float)
F64P = POINTER(c_double)


def build(ref: bool = True) -> None:
    """Build the oracle (and, where the reference tree exists, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref"], check=True)


def gold_lib() -> ctypes.CDLL:
    global _gold
    if _gold is None:
        path = BUILD / "libgold.so"
        if not path.exists():
            build(ref=False)
        lib = ctypes.CDLL(str(path))
        for suf, P, T in (("f32", F32P, c_float), ("f64", F64P, c_double)):
            for nm in ("gold_serial", "gold_test_generation"):
                getattr(lib, f"{nm}_{suf}").restype = None
            getattr(lib, f"gold_serial_{suf}").argtypes = [P, P, P, P, P, c_int]
            getattr(lib, f"gold_many_systems_{suf}").argtypes = [P, P, P, P, P, c_int, c_int]
            getattr(lib, f"gold_multithread_many_systems_{suf}").argtypes = [P, P, P, P, P, c_int, c_int]
            getattr(lib, f"gold_many_systems_omp_{suf}").argtypes = [P, P, P, P, P, c_int, c_int, c_int]
            getattr(lib, f"gold_test_generation_{suf}").argtypes = [P, P, P, P, P, c_int]
            getattr(lib, f"gold_compare_{suf}").argtypes = [P, P, c_int]
            getattr(lib, f"gold_compare_{suf}").restype = T
            getattr(lib, f"gold_compare_many_systems_{suf}").argtypes = [P, P, c_int, c_int, T, P]
            getattr(lib, f"gold_compare_many_systems_{suf}").restype = c_int
        lib.gold_srand.argtypes = [c_uint]
        lib.gold_max_threads.restype = c_int
        lib.gold_solve_f64_from_f32.argtypes = [F32P, F32P, F32P, F32P, F64P, c_int, c_int, c_int, c_int]
        lib.gold_rel_residual.argtypes = [F32P, F32P, F32P, F32P, F64P, F32P, c_int, c_int, c_int, F64P, c_int]
        lib.gold_check_ragged.argtypes = [F32P, F32P, F32P, F32P, F64P, F32P, POINTER(ctypes.c_long), c_int, F64P,
                                          F64P, F64P, c_int]
        _gold = lib
    return _gold


def ref_gold_lib(prec: str) -> ctypes.CDLL | None:
    """The reference's own tridiagonal_gold.h routines (None if not built here)."""
    if prec not in _ref:
        path = REF / f"libgold_ref_{prec}.so"
        if not path.exists():
            _ref[prec] = None
        else:
            lib = ctypes.CDLL(str(path))
            P = F32P if prec == "f32" else F64P
            getattr(lib, f"ref_serial_many_systems_{prec}").argtypes = [P, P, P, P, P, c_int, c_int]
            getattr(lib, f"ref_multithread_many_systems_{prec}").argtypes = [P, P, P, P, P, c_int, c_int]
            getattr(lib, f"ref_test_generation_{prec}").argtypes = [P, P, P, P, P, c_int]
            getattr(lib, f"ref_srand_{prec}").argtypes = [c_uint]
            _ref[prec] = lib
    return _ref[prec]


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(F32P if a.dtype == np.float32 else F64P)


def _suf(dtype) -> str:
    return "f32" if np.dtype(dtype) == np.float32 else "f64"


def generate_reference_inputs(n: int, m: int, dtype=np.float32, seed: int = 1, use_ref: bool = False):
    """The reference's generator (tridiagonal_gold.h:81-94) for m systems of size
    n, after srand(seed): returns (a, b, c, d) as (m, n) arrays."""
    suf = _suf(dtype)
    arrs = [np.zeros((m, n), dtype) for _ in range(5)]
    if use_ref:
        lib = ref_gold_lib(suf)
        getattr(lib, f"ref_srand_{suf}")(seed)
        gen = getattr(lib, f"ref_test_generation_{suf}")
    else:
        lib = gold_lib()
        lib.gold_srand(seed)
        gen = getattr(lib, f"gold_test_generation_{suf}")
    for i in range(m):
        gen(*[_ptr(x[i]) for x in arrs], n)
    return tuple(arrs[:4])


def serial_many(a, b, c, d, *, use_ref: bool = False, threads: int | None = None):
    """The gold Thomas solver of tridiagonal_gold.h:26-53 in the inputs' precision.
    Works on copies (the reference overwrites c and d).  threads=None: one core
    (serialManySystems); threads=k: gold_many_systems_omp with k threads."""
    suf = _suf(a.dtype)
    m, n = a.shape
    a2, b2, c2, d2 = (np.ascontiguousarray(v).copy() for v in (a, b, c, d))
    x = np.zeros_like(a2)
    if use_ref:
        getattr(ref_gold_lib(suf), f"ref_serial_many_systems_{suf}")(*map(_ptr, (a2, b2, c2, d2, x)), n, m)
    elif threads is None:
        getattr(gold_lib(), f"gold_many_systems_{suf}")(*map(_ptr, (a2, b2, c2, d2, x)), n, m)
    else:
        getattr(gold_lib(), f"gold_many_systems_omp_{suf}")(*map(_ptr, (a2, b2, c2, d2, x)), n, m, threads)
    return x


def multithread_many(a, b, c, d, *, use_ref: bool = False):
    """tridiagonal_gold.h:56-72 (4 threads; the m % 4 trailing systems stay 0)."""
    suf = _suf(a.dtype)
    m, n = a.shape
    a2, b2, c2, d2 = (np.ascontiguousarray(v).copy() for v in (a, b, c, d))
    x = np.zeros_like(a2)
    lib = ref_gold_lib(suf) if use_ref else gold_lib()
    fn = getattr(lib, f"ref_multithread_many_systems_{suf}") if use_ref else getattr(lib, f"gold_multithread_many_systems_{suf}")
    fn(*map(_ptr, (a2, b2, c2, d2, x)), n, m)
    return x


def solve_f64(a, b, c, d, layout: int = 0, threads: int = 0) -> np.ndarray:
    """Strict oracle: gold Thomas in FP64 on FP32 inputs.  Arrays are (m, n) for
    layout 0 (contiguous) or (n, m) for layout 1 (interleaved)."""
    a, b, c, d = (np.ascontiguousarray(v, dtype=np.float32) for v in (a, b, c, d))
    if layout == 0:
        m, n = a.shape
    else:
        n, m = a.shape
    x = np.zeros(a.shape, np.float64)
    gold_lib().gold_solve_f64_from_f32(*map(_ptr, (a, b, c, d, x)), n, m, layout, threads)
    return x


def rel_residual(a, b, c, d, x, layout: int = 0, threads: int = 0) -> np.ndarray:
    """Per system ||d - T x|| / ||d|| evaluated in FP64 (x FP32 or FP64)."""
    a, b, c, d = (np.ascontiguousarray(v, dtype=np.float32) for v in (a, b, c, d))
    if layout == 0:
        m, n = a.shape
    else:
        n, m = a.shape
    out = np.zeros(m, np.float64)
    lib = gold_lib()
    if x.dtype == np.float64:
        x = np.ascontiguousarray(x)
        lib.gold_rel_residual(*map(_ptr, (a, b, c, d)), _ptr(x), None, n, m, layout, _ptr(out), threads)
    else:
        x = np.ascontiguousarray(x, dtype=np.float32)
        lib.gold_rel_residual(*map(_ptr, (a, b, c, d)), None, _ptr(x), n, m, layout, _ptr(out), threads)
    return out


def check_ragged(a, b, c, d, x, offsets, threads: int = 0):
    """Ragged batch (system s = rows offsets[s]..offsets[s+1] of the 1-D
    arrays): per system the FP64 relative residual of x (FP32 or FP64) and
    its forward error against the FP64 gold solution.  Returns (res, fwd)."""
    a, b, c, d = (np.ascontiguousarray(v, dtype=np.float32) for v in (a, b, c, d))
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    m = len(off) - 1
    total = int(off[-1])
    res = np.zeros(m, np.float64)
    fwd = np.zeros(m, np.float64)
    x = np.ascontiguousarray(x)
    assert x.size >= total and a.size >= total
    x64p = _ptr(x) if x.dtype == np.float64 else None
    x32p = _ptr(np.ascontiguousarray(x, dtype=np.float32)) if x.dtype != np.float64 else None
    gold_lib().gold_check_ragged(*map(_ptr, (a, b, c, d)), x64p, x32p,
                                 off.ctypes.data_as(POINTER(ctypes.c_long)), m, None, _ptr(res), _ptr(fwd), threads)
    return res, fwd


def compare_many(x1, x2, eps):
    """compareManySystems (tridiagonal_gold.h:133-148): (#failed, per-system RMS)."""
    suf = _suf(x1.dtype)
    m, n = x1.shape
    rms = np.zeros(m, x1.dtype)
    T = c_float if suf == "f32" else c_double
    nf = getattr(gold_lib(), f"gold_compare_many_systems_{suf}")(
        _ptr(np.ascontiguousarray(x1)), _ptr(np.ascontiguousarray(x2)), n, m, T(eps), _ptr(rms)
    )
    return nf, rms


# ---- the reference's own GPU kernels ------------------------------------------
class RefKernels:
    """Launches the reference kernels from oracle/_ref cubins on device buffers
    (torch tensors).  The reference kernels overwrite a, b, c, d."""

    KIND = {"cr": 0, "pcr": 1, "crpcr": 2, "crNBC": 3, "crpcrNBC": 4, "crNBC32": 5}

    def __init__(self):
        global _runner
        if _runner is None:
            path = BUILD / "libref_runner.so"
            if not path.exists():
                build(ref=False)
            lib = ctypes.CDLL(str(path))
            lib.refk_init.argtypes = [ctypes.c_char_p]
            lib.refk_solve.argtypes = [c_int, c_int] + [c_void_p] * 5 + [c_int, c_int, c_int, c_void_p]
            lib.refk_pcr_gauss.argtypes = [c_int] + [c_void_p] * 8 + [c_int, c_int, c_int, c_void_p, POINTER(c_int)]
            lib.refk_last_error.restype = ctypes.c_char_p
            _runner = lib
        self.lib = _runner
        if not (REF / "f32" / "cr_app.cubin").exists():
            raise FileNotFoundError("reference kernels were not built (oracle/_ref/f32/*.cubin missing)")
        self._check(self.lib.refk_init(str(REF).encode()), "refk_init")

    @staticmethod
    def available() -> bool:
        return (REF / "f32" / "cr_app.cubin").exists()

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: {self.lib.refk_last_error().decode()} (rc {rc})")

    def solve(self, kind, a, b, c, d, x, n, m, rest=0, stream=0):
        import torch

        dbl = int(a.dtype == torch.float64)
        self._check(
            self.lib.refk_solve(self.KIND[kind], dbl, a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(),
                                x.data_ptr(), n, m, rest, c_void_p(stream)),
            f"reference {kind}",
        )

    def pcr_gauss(self, a, b, c, d, a2, b2, c2, d2, n, m, g, stream=0) -> int:
        """Returns 1 if the solution is left in d2, else 0 (it is in d)."""
        import torch

        dbl = int(a.dtype == torch.float64)
        which = c_int(0)
        self._check(
            self.lib.refk_pcr_gauss(dbl, *(t.data_ptr() for t in (a, b, c, d, a2, b2, c2, d2)), n, m, g,
                                    c_void_p(stream), ctypes.byref(which)),
            "reference pcrGauss",
        )
        return which.value
