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
