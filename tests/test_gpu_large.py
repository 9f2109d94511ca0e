"""GPU parity of the large-system solver (tridi_solve_large_*), contiguous and
interleaved layouts, against the FP64 oracle.  Tolerances: tests/parity.py;
the weakly dominant systems (b = |a|+|c|+U[0.01,0.1]) are ill-conditioned
enough that FP32 results are held to a residual of 1e-5 and a forward error
of 5e-3 (the FP32 gold solver's own errors are of that order)."""
import numpy as np
import pytest

import tridiagonalsolvers_gb300 as tg
from oracle import gold
from tridiagonalsolvers_gb300 import workloads

from .parity import check_against_oracle

pytestmark = pytest.mark.gpu
NP = {"f32": np.float32, "f64": np.float64}
WEAK = dict(res_tol=1e-5, fwd_tol=5e-3)


def _dev(cuda, *arrs):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(v).ravel()).to(cuda) for v in arrs]


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n,m", [(1, 7), (15, 9), (16, 9), (17, 33), (1000, 64), (4096, 100), (20000, 3)])
def test_large_interleaved(cuda, n, m, prec):
    dt = NP[prec]
    a, b, c, d = workloads.dominant(m, n, seed=n + m, dtype=dt, layout=1)  # (n, m) arrays
    x = tg.solve_large(*_dev(cuda, a, b, c, d), n, m, "interleaved").cpu().numpy().reshape(n, m)
    assert tg.device_status() == 0
    check_against_oracle(a, b, c, d, x, layout=1, dtype=dt)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n,m", [(5, 4), (1000, 7), (30000, 2), (65536, 3)])
def test_large_contiguous(cuda, n, m, prec):
    dt = NP[prec]
    a, b, c, d = workloads.dominant(m, n, seed=3 * n + m, dtype=dt)
    x = tg.solve_large(*_dev(cuda, a, b, c, d), n, m, "contiguous").cpu().numpy().reshape(m, n)
    check_against_oracle(a, b, c, d, x, dtype=dt)


def test_large_weak_interleaved(cuda):
    n, m = 8192, 128
    a, b, c, d = workloads.weak(m, n, seed=1003, layout=1)
    x = tg.solve_large(*_dev(cuda, a, b, c, d), n, m, "interleaved").cpu().numpy().reshape(n, m)
    check_against_oracle(a, b, c, d, x, layout=1, **WEAK)


def test_large_full_size_1024x65536_interleaved(cuda):
    """The large-system workload at full size: 1024 systems x 65536 unknowns,
    interleaved, weakly dominant.  Sampled systems are checked against the
    FP64 oracle; every entry must be finite."""
    import torch

    n, m = 65536, 1024
    a, b, c, d = workloads.weak(m, n, seed=workloads.SEEDS["c3"], layout=1)
    ta, tb, tc, td = _dev(cuda, a, b, c, d)
    x = tg.solve_large(ta, tb, tc, td, n, m, "interleaved")
    assert bool(torch.isfinite(x).all())
    cols = np.array([0, 1, 31, 32, 511, 1000, 1023])
    xs = x.view(n, m)[:, cols].cpu().numpy()
    check_against_oracle(a[:, cols], b[:, cols], c[:, cols], d[:, cols], xs, layout=1, **WEAK)


@pytest.mark.parametrize("n,m", [(5000, 64), (65536, 32), (300, 96), (20000, 48)])
def test_large_interleaved_tma_passes_match_register_passes(cuda, n, m):
    """Interleaved FP32 with m a multiple of 32 runs the TMA-tiled reduce and
    back passes; they agree with the register-kernel passes (forced with
    TRIDI_TUNE_LARGE_TMA = 2) and with the FP64 oracle.  m = 48 takes the
    register passes either way."""
    import torch

    from tridiagonalsolvers_gb300 import _lib

    L = _lib.lib()
    a, b, c, d = workloads.weak(m, n, seed=n + m, layout=1)
    t = [torch.from_numpy(np.ascontiguousarray(v).ravel()).to(cuda) for v in (a, b, c, d)]
    outs = []
    for mode in (0, 2):
        L.tridi_set_tunable(6, mode)
        try:
            outs.append(tg.solve_large(*t, n, m, layout="interleaved").cpu().numpy())
        finally:
            L.tridi_set_tunable(6, 0)
    x_tma, x_reg = outs
    scale = np.abs(x_reg).max()
    assert np.abs(x_tma - x_reg).max() <= 1e-5 * scale
    xs = x_tma.reshape(n, m)
    res = gold.rel_residual(a, b, c, d, xs, layout=1)
    assert res.max() <= 1e-5, f"residual {res.max():.2e}"
