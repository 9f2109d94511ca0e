"""GPU parity of mixed-precision iterative refinement (tridi_refine_f32, the
residual and update in double-float or native FP64) against the FP64 oracle:
the refined FP64 solution must reach a relative residual of 1e-10 (the stated
target) and agree with the oracle's FP64 solution; the number of correction
sweeps is recorded."""
import numpy as np
import pytest

import tridiagonalsolvers_gb300 as tg
from oracle import gold
from tridiagonalsolvers_gb300 import workloads

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _dev(cuda, *arrs):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(v).ravel()).to(cuda) for v in arrs]


def _check(a, b, c, d, x, layout, sweeps, rel):
    res = gold.rel_residual(a, b, c, d, x, layout=layout)
    assert res.max() <= 1.5 * TOL, f"oracle residual {res.max():.3e} after {sweeps} sweeps (kernel said {rel:.3e})"
    x64 = gold.solve_f64(a, b, c, d, layout=layout)
    ax = 1 if layout == 0 else 0
    fwd = (np.abs(x - x64).max(axis=ax) / np.abs(x64).max(axis=ax)).max()
    assert fwd < 1e-7, f"forward error vs FP64 oracle {fwd:.3e}"
    print(f"sweeps={sweeps} residual={res.max():.2e} fwd={fwd:.2e}")


@pytest.mark.parametrize("residual", ["df", "fp64"])
@pytest.mark.parametrize("n,m", [(256, 64), (512, 33), (1000, 17), (4096, 8), (20000, 2)])
def test_refine_contiguous_dominant(cuda, n, m, residual):
    a, b, c, d = workloads.dominant(m, n, seed=n + m)
    x, sweeps, rel = tg.refine(*_dev(cuda, a, b, c, d), n, m, tol=TOL, residual=residual)
    _check(a, b, c, d, x.cpu().numpy().reshape(m, n), 0, sweeps, rel)
    assert 1 <= sweeps <= 4


@pytest.mark.parametrize("residual", ["df", "fp64"])
@pytest.mark.parametrize("n,m", [(1024, 64), (8192, 96)])
def test_refine_interleaved_weak(cuda, n, m, residual):
    a, b, c, d = workloads.weak(m, n, seed=1003 + n, layout=1)
    x, sweeps, rel = tg.refine(*_dev(cuda, a, b, c, d), n, m, layout="interleaved", tol=TOL, max_sweeps=20,
                               residual=residual)
    _check(a, b, c, d, x.cpu().numpy().reshape(n, m), 1, sweeps, rel)


def test_refine_adi_lines(cuda):
    sizes = np.full(40, 3000)
    a, b, c, d, _ = workloads.adi(sizes, seed=4)
    shp = (40, 3000)
    a, b, c, d = (v.reshape(shp) for v in (a, b, c, d))
    x, sweeps, rel = tg.refine(*_dev(cuda, a, b, c, d), 3000, 40, tol=TOL)
    _check(a, b, c, d, x.cpu().numpy().reshape(shp), 0, sweeps, rel)


def test_refine_reports_non_convergence(cuda):
    a, b, c, d = workloads.weak(4, 4096, seed=9)
    with pytest.raises(tg.TridiError) as ei:
        tg.refine(*_dev(cuda, a, b, c, d), 4096, 4, tol=1e-30, max_sweeps=1)
    assert ei.value.status == 6


@pytest.mark.parametrize("residual", ["df", "fp64"])
def test_refine_full_size_1024x65536_interleaved(cuda, residual):
    """The large-system workload with refinement to 1e-10: sampled systems are
    checked against the FP64 oracle."""
    import torch

    n, m = 65536, 1024
    a, b, c, d = workloads.weak(m, n, seed=workloads.SEEDS["c3"], layout=1)
    x, sweeps, rel = tg.refine(*_dev(cuda, a, b, c, d), n, m, layout="interleaved", tol=TOL, max_sweeps=20,
                               residual=residual)
    assert bool(torch.isfinite(x).all())
    cols = np.array([0, 5, 500, 1023])
    xs = x.view(n, m)[:, cols].cpu().numpy()
    _check(a[:, cols], b[:, cols], c[:, cols], d[:, cols], xs, 1, sweeps, rel)
    print(f"1024x65536 interleaved weak: {sweeps} sweeps to {rel:.2e}")


@pytest.mark.parametrize("residual", ["df", "fp64"])
@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("max_sweeps", [0, 1, 2, 3])
def test_refine_every_sweep_count(cuda, residual, layout, max_sweeps):
    """An unreachable tolerance runs exactly max_sweeps corrections and
    reports non-convergence; x is still the refined solution of that many
    sweeps (FP32-level after none, at the 1e-10 level after one or more) --
    every path of the sweep sequence (first sweep only, the FP64 write of the
    second, pairs again from the third) ends with x in FP64."""
    import ctypes

    import torch

    from tridiagonalsolvers_gb300 import _lib

    n, m = (1000, 17) if layout == 0 else (2048, 64)
    a, b, c, d = workloads.dominant(m, n, seed=31 + max_sweeps, layout=layout)
    t = _dev(cuda, a, b, c, d)
    x = torch.full((n * m,), float("nan"), dtype=torch.float64, device=cuda)
    L = _lib.lib()
    wsb = L.tridi_refine_workspace_bytes(n, m, layout)
    ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
    sweeps, rel = ctypes.c_int(-1), ctypes.c_double(0.0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    prev = L.tridi_get_tunable(4)
    L.tridi_set_tunable(4, {"df": 1, "fp64": 2}[residual])
    try:
        st = L.tridi_refine_f32(*(v.data_ptr() for v in t), x.data_ptr(), n, m, layout, 1e-30, max_sweeps,
                                ws.data_ptr(), wsb, stream, ctypes.byref(sweeps), ctypes.byref(rel))
    finally:
        L.tridi_set_tunable(4, prev)
    torch.cuda.synchronize()
    assert st == 6 and sweeps.value == max_sweeps  # TRIDI_ERROR_NOT_CONVERGED after max_sweeps corrections
    shp = (m, n) if layout == 0 else (n, m)
    xs = x.cpu().numpy().reshape(shp)
    assert np.all(np.isfinite(xs))
    res = gold.rel_residual(a, b, c, d, xs, layout=layout)
    if max_sweeps == 0:
        assert res.max() <= 2e-6
    else:
        assert res.max() <= TOL, f"{max_sweeps} sweeps: oracle residual {res.max():.2e}"
    # the kernel's own maximum agrees with the oracle's (both near the floor
    # of the residual arithmetic after two or three sweeps)
    assert rel.value <= 4 * res.max() + 1e-13 and res.max() <= 4 * rel.value + 1e-13
