"""Shared parity checks: a GPU result against the FP64 oracle and against the
reference's own FP32/FP64 kernels.

Tolerances (stated once, used by every GPU parity test):
  * FP64 oracle (gold Thomas in FP64 on the same inputs, oracle/gold.c):
      relative residual ||d - T x|| / ||d||  <= RES_TOL[dtype] per system
      forward error max|x - x64| / max|x64|  <= FWD_TOL[dtype] per system
  * reference kernels (the reference's own CUDA kernels rebuilt for sm_103a):
      |x - x_ref| <= ULP_TOL * ulp(max |x_ref|) per system,
    i.e. agreement to within 64 units in the last place of the system's
    largest unknown.
  * legacy acceptance of the reference driver (test_tridiagonal.cpp:107):
      compareManySystems against the gold solver at eps = 1e-3 -> 0 failures.
"""
from __future__ import annotations

import numpy as np

from oracle import gold

RES_TOL = {np.float32: 2e-6, np.float64: 1e-14}
FWD_TOL = {np.float32: 2e-5, np.float64: 1e-12}
ULP_TOL = 64


def check_against_oracle(a, b, c, d, x, layout=0, dtype=np.float32, res_tol=None, fwd_tol=None, x64=None):
    """a..d, x are host numpy arrays; returns (max residual, max fwd error).
    Every system is checked.  x64: the oracle's FP64 solution of these FP32
    inputs when the caller already has it (several solvers checked against
    one batch), else computed here."""
    a32, b32, c32, d32 = (np.asarray(v, np.float32) for v in (a, b, c, d))
    if dtype == np.float64:
        # FP64 inputs: residual and oracle computed from FP64 data directly.
        res, fwd = _f64_metrics(a, b, c, d, x, layout)
    else:
        if x64 is None:
            x64 = gold.solve_f64(a32, b32, c32, d32, layout=layout)
        res = gold.rel_residual(a32, b32, c32, d32, np.asarray(x), layout=layout)
        ax = 1 if layout == 0 else 0
        err = np.abs(np.asarray(x, np.float64) - x64).max(axis=ax)
        scale = np.abs(x64).max(axis=ax)
        fwd = err / np.where(scale > 0, scale, 1.0)
    res_tol = RES_TOL[dtype] if res_tol is None else res_tol
    fwd_tol = FWD_TOL[dtype] if fwd_tol is None else fwd_tol
    assert np.all(np.isfinite(x)), "non-finite entries in the solution"
    assert res.max() <= res_tol, f"relative residual {res.max():.3e} > {res_tol:.1e}"
    assert fwd.max() <= fwd_tol, f"forward error {fwd.max():.3e} > {fwd_tol:.1e}"
    return float(res.max()), float(fwd.max())


def _f64_metrics(a, b, c, d, x, layout):
    if layout == 1:
        a, b, c, d, x = (np.ascontiguousarray(np.asarray(v).T) for v in (a, b, c, d, x))
    x64 = gold.serial_many(*(np.asarray(v, np.float64) for v in (a, b, c, d)))
    r = np.array(d, np.float64) - b * x
    r[:, 1:] -= a[:, 1:] * x[:, :-1]
    r[:, :-1] -= c[:, :-1] * x[:, 1:]
    res = np.linalg.norm(r, axis=1) / np.maximum(np.linalg.norm(d, axis=1), 1e-300)
    fwd = np.abs(x - x64).max(axis=1) / np.maximum(np.abs(x64).max(axis=1), 1e-300)
    return res, fwd


def check_ulps(x, x_ref, ulps=ULP_TOL):
    """Per system |x - x_ref| <= ulps * ulp(max |x_ref|); rows are systems."""
    x = np.asarray(x)
    x_ref = np.asarray(x_ref)
    big = np.abs(x_ref).max(axis=1)
    ulp = np.spacing(big.astype(x_ref.dtype)).astype(np.float64)
    diff = np.abs(x.astype(np.float64) - x_ref.astype(np.float64)).max(axis=1)
    worst = float((diff / ulp).max())
    assert worst <= ulps, f"differs from the reference kernel by {worst:.1f} ulp (> {ulps})"
    return worst


def check_ulps_where_reference_valid(x, x_ref, a, b, c, d, dtype=np.float32, ulps=ULP_TOL):
    """check_ulps on the systems whose reference-kernel result itself passes the
    oracle's residual bound; returns (#systems compared, #reference failures).

    Where the reference kernel's own answer does not solve the system, the
    comparison is meaningless; those systems are excluded here (the product
    result is checked against the FP64 oracle regardless).  Observed on
    sm_103a: the FP64 builds of crKernel and pcrKernel leave systems of 16
    unknowns unsolved.  Both take their level count from
    (int)log2(T(systemSize/2)) (cr_kernel.cu:11, pcr_kernel.cu:7).  By code
    reading, cr / crNBC also lack a barrier between the last forward level and
    the 2x2 solve (cr_kernel.cu:41-63, crNBC.cu:52-78)."""
    x_ref = np.asarray(x_ref)
    if dtype == np.float64:
        res, _ = _f64_metrics(a, b, c, d, x_ref, 0)
    else:
        res = gold.rel_residual(*(np.asarray(v, np.float32) for v in (a, b, c, d)), x_ref)
    ok = res <= RES_TOL[dtype]
    if ok.any():
        check_ulps(np.asarray(x)[ok], x_ref[ok], ulps)
    return int(ok.sum()), int((~ok).sum())


def legacy_accept(x, a, b, c, d):
    """The reference driver's own acceptance: RMS vs gold <= 1e-3 for every
    system, with the gold solver and the comparison in the inputs' precision
    (float, or double in the reference's USE_DOUBLE build)."""
    dt = np.float64 if np.asarray(a).dtype == np.float64 else np.float32
    x_gold = gold.serial_many(*(np.asarray(v, dt) for v in (a, b, c, d)))
    nf, _ = gold.compare_many(np.asarray(x, dt), x_gold, 1e-3)
    assert nf == 0, f"{nf} systems fail the reference's 1e-3 RMS acceptance"
