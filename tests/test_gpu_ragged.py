"""GPU parity of the ragged persistent solver (tridi_ragged_*) against the
FP64 oracle, system by system.  Tolerances: tests/parity.py."""
import numpy as np
import pytest

from oracle import gold
from tridiagonalsolvers_gb300 import workloads
from tridiagonalsolvers_gb300.ragged import RaggedPlan, padded

from .parity import RES_TOL

pytestmark = pytest.mark.gpu


def _dev(cuda, v, total):
    import torch

    t = torch.zeros(padded(total), dtype=torch.float32, device=cuda)
    t[:total] = torch.from_numpy(v)
    return t


def _check_systems(a, b, c, d, x, off, idx, res_tol=RES_TOL[np.float32], fwd_tol=2e-5):
    for s in idx:
        lo, hi = off[s], off[s + 1]
        sl = [v[lo:hi][None] for v in (a, b, c, d)]
        xs = x[lo:hi][None]
        res = gold.rel_residual(*sl, xs)[0]
        x64 = gold.solve_f64(*sl)[0]
        fwd = np.abs(xs[0] - x64).max() / np.abs(x64).max()
        assert res <= res_tol and fwd <= fwd_tol, f"system {s} (n={hi - lo}): residual {res:.2e} fwd {fwd:.2e}"


@pytest.mark.parametrize("seed", [1, 2])
def test_ragged_mixed_sizes(cuda, seed):
    rng = np.random.default_rng(seed)
    sizes = np.concatenate([rng.integers(1, 40, 50), rng.integers(40, 481, 300), rng.integers(481, 6000, 40),
                            rng.integers(6000, 8705, 12), [1, 2, 3, 480, 481, 6141, 6144, 8704]])
    rng.shuffle(sizes)
    a, b, c, d, off = workloads.adi(sizes, seed=seed)
    total = int(off[-1])
    plan = RaggedPlan(off)
    x = plan.solve(*(_dev(cuda, v, total) for v in (a, b, c, d))).cpu().numpy()[:total]
    _check_systems(a, b, c, d, x, off, range(len(sizes)))
    # replaying the plan gives the same answer bit for bit
    x2 = plan.solve(*(_dev(cuda, v, total) for v in (a, b, c, d))).cpu().numpy()[:total]
    assert np.array_equal(x, x2)


def test_ragged_alone_equals_in_batch(cuda):
    """Each system's solution does not depend on what else is in the batch."""
    sizes = np.array([700, 33, 5000, 129, 8192, 64])
    a, b, c, d, off = workloads.adi(sizes, seed=9)
    total = int(off[-1])
    xb = RaggedPlan(off).solve(*(_dev(cuda, v, total) for v in (a, b, c, d))).cpu().numpy()
    for s in range(len(sizes)):
        lo, hi = off[s], off[s + 1]
        o1 = np.array([0, hi - lo])
        xs = RaggedPlan(o1).solve(*(_dev(cuda, v[lo:hi], hi - lo) for v in (a, b, c, d))).cpu().numpy()
        assert np.array_equal(xs[: hi - lo], xb[lo:hi])


def test_ragged_full_workload_100000_systems(cuda):
    """100000 ADI systems, sizes log-uniform in [32, 8192]: every system's
    residual is checked on a sample, every entry must be finite."""
    sizes = workloads.ragged_sizes(100000, 32, 8192, seed=workloads.SEEDS["c4"])
    a, b, c, d, off = workloads.adi(sizes, seed=workloads.SEEDS["c4"])
    total = int(off[-1])
    plan = RaggedPlan(off)
    x = plan.solve(*(_dev(cuda, v, total) for v in (a, b, c, d))).cpu().numpy()[:total]
    assert np.all(np.isfinite(x))
    rng = np.random.default_rng(0)
    _check_systems(a, b, c, d, x, off, rng.choice(len(sizes), 300, replace=False))
