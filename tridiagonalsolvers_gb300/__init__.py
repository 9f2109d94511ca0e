"""GB300-native batched tridiagonal solvers (sm_103a CUDA behind a C ABI).

The reference's solvers, with the reference's names, on device tensors:

    cr(a, b, c, d)                 cyclic reduction              (cr_app.cu:4)
    pcr(a, b, c, d)                parallel cyclic reduction      (pcr_app.cu:5)
    crpcr(a, b, c, d, rest)        hybrid CR-PCR                  (crpcr_app.cu:5)
    crNBC / crNBC32 / crpcrNBC     bank-conflict-free shared CR   (crNBC.cu, crNBC32banks.cu)
    pcrGauss(a, b, c, d, g)        PCR-then-Thomas, g chains      (pcrGauss_app.cu:164)
    solve(a, b, c, d)              any-size partition solver      (GB300 addition)
    solve_large(..., layout)       large / interleaved systems    (GB300 addition)
    refine(..., tol)               FP32 solves + FP64 residual    (GB300 addition)

Each takes CUDA tensors shaped (num_systems, system_size) (or flat with an
explicit system_size) of float32 or float64, returns x, and launches on the
current torch stream.  PyTorch is used only for device memory and streams;
the work is done by the native library through its C ABI (include/tridi.h).
"""
from __future__ import annotations

from ._lib import TridiError, lib  # noqa: F401
from .solvers import (  # noqa: F401
    cr,
    crNBC,
    crNBC32,
    crpcr,
    crpcrNBC,
    device_status,
    pcr,
    pcrGauss,
    refine,
    solve,
    solve_large,
)

__all__ = ["cr", "pcr", "crpcr", "crNBC", "crNBC32", "crpcrNBC", "pcrGauss", "solve", "solve_large", "refine", "device_status", "TridiError", "lib"]
