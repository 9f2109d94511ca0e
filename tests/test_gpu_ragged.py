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
                            rng.integers(6000, 12281, 12),
                            [1, 2, 3, 480, 481, 2400, 2401, 6141, 6144, 8704, 12279, 12280]])
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


@pytest.mark.parametrize("residual", ["df", "fp64"])
def test_ragged_refined_graph_replay(cuda, residual):
    """Fused refinement of a ragged batch (every item kind: warp, 160-thread
    group, whole CTA in the ring, and systems beyond the ring refined from
    global memory, up to 24480 rows; 13000 and 13560 rows fit the ring of the
    one-correction form only) to 1e-10, captured once in a CUDA graph;
    replays agree bit for bit with the eager launch and with the FP64 oracle."""
    from tridiagonalsolvers_gb300.ragged import RaggedRefiner

    rng = np.random.default_rng(3)
    sizes = np.concatenate([rng.integers(32, 480, 200), rng.integers(480, 12280, 40), rng.integers(12281, 24481, 6),
                            [13000, 13560, 16384, 24480]])
    a, b, c, d, off = workloads.adi(sizes, seed=5)
    total = int(off[-1])
    t = [_dev(cuda, v, total) for v in (a, b, c, d)]
    plan = RaggedPlan(off)
    eager = RaggedRefiner(plan, *t, sweeps=1, graph=False, residual=residual)
    xe, rel_e = eager.run()
    xe = xe.cpu().numpy()[:total].copy()
    g = RaggedRefiner(plan, *t, sweeps=1, graph=True, residual=residual)
    for _ in range(2):
        xg, rel_g = g.run()
        assert np.array_equal(xg.cpu().numpy()[:total], xe)
        assert rel_g == rel_e
    assert rel_e <= 1e-10, f"max relative residual {rel_e:.2e} after one sweep"
    worst = 0.0
    for s in range(len(sizes)):
        lo, hi = off[s], off[s + 1]
        sl = [v[lo:hi][None] for v in (a, b, c, d)]
        res = gold.rel_residual(*sl, xe[lo:hi][None])[0]
        worst = max(worst, res)
        assert res <= 1e-10, f"system {s} (n={hi - lo}) oracle residual {res:.2e}"
        x64 = gold.solve_f64(*sl)[0]
        fwd = np.abs(xe[lo:hi] - x64).max() / np.abs(x64).max()
        assert fwd <= 1e-9, f"system {s} (n={hi - lo}) forward error {fwd:.2e}"
    # the device's own maximum agrees with the oracle's to a few digits
    assert rel_e <= 2 * worst + 1e-15 and worst <= 2 * rel_e + 1e-15


@pytest.mark.parametrize("residual", ["df", "fp64"])
@pytest.mark.parametrize("sweeps", [0, 2])
def test_ragged_refined_sweeps(cuda, residual, sweeps):
    """Zero sweeps leaves the FP32 solution (widened) with its FP32-level
    residual; two sweeps stay at the 1e-10 level."""
    from tridiagonalsolvers_gb300.ragged import RaggedRefiner

    sizes = np.array([64, 300, 1000, 2400, 5000, 9000, 9300, 15000, 33, 480, 481, 2401])
    a, b, c, d, off = workloads.adi(sizes, seed=21)
    total = int(off[-1])
    t = [_dev(cuda, v, total) for v in (a, b, c, d)]
    x, rel = RaggedRefiner(RaggedPlan(off), *t, sweeps=sweeps, graph=False, residual=residual).run()
    x = x.cpu().numpy()[:total]
    for s in range(len(sizes)):
        lo, hi = off[s], off[s + 1]
        sl = [v[lo:hi][None] for v in (a, b, c, d)]
        res = gold.rel_residual(*sl, x[lo:hi][None])[0]
        if sweeps == 0:
            assert res <= RES_TOL[np.float32], f"system {s} (n={hi - lo}) residual {res:.2e}"
        else:
            assert res <= 1e-10, f"system {s} (n={hi - lo}) residual {res:.2e}"


def test_ragged_big_systems_plain(cuda):
    sizes = np.array([12281, 12000, 16384, 17408, 24480, 100, 9000, 20001])
    a, b, c, d, off = workloads.adi(sizes, seed=8)
    total = int(off[-1])
    x = RaggedPlan(off).solve(*(_dev(cuda, v, total) for v in (a, b, c, d))).cpu().numpy()[:total]
    _check_systems(a, b, c, d, x, off, range(len(sizes)))


def test_ragged_rejects_oversize_systems():
    from tridiagonalsolvers_gb300 import _lib

    with pytest.raises(_lib.TridiError):
        RaggedPlan(np.array([0, 100, 100 + 24481]))


def test_double_float_to_fp64_is_correctly_rounded(cuda):
    """The refinement's FP64 output assembly (scaled-conversion fast path +
    FP64 add fallback) equals numpy's correctly rounded float64(hi) +
    float64(lo) for normalised pairs, including lo finer than hi's double ulp,
    exact ties at a half and a quarter of that ulp, hi a power of two with lo
    of the opposite sign, zeros, tiny hi and subnormal lo."""
    import ctypes

    import torch

    from tridiagonalsolvers_gb300 import _lib

    rng = np.random.default_rng(5)
    n = 1 << 20
    hi = (rng.standard_normal(n) * 10.0 ** rng.integers(-20, 20, n)).astype(np.float32)
    hi[:4096] = np.float32(2.0) ** rng.integers(-60, 60, 4096)  # powers of two
    hi[4096:4200] = 0.0
    # lo within half an ulp of hi, at every scale below it
    ulp = np.spacing(np.abs(hi)).astype(np.float64)
    frac = rng.uniform(-0.5, 0.5, n) * 2.0 ** -rng.integers(0, 40, n).astype(np.float64)
    lo = (frac * ulp).astype(np.float32)
    lo[::7] = 0.0
    lo[4200:4300] = np.float32(1e-42)  # subnormal
    # ties: odd multiples of a half, quarter or eighth of hi's double ulp
    k = 20000
    du = np.spacing(np.abs(hi[5000:5000 + k]).astype(np.float64)) * 2.0 ** -29
    odd = (2 * rng.integers(1, 1 << 20, k) + 1).astype(np.float64)
    tie = odd * du * 2.0 ** -rng.integers(1, 4, k).astype(np.float64) * rng.choice([-1.0, 1.0], k)
    tf = tie.astype(np.float32)
    lo[5000:5000 + k] = np.where(tf.astype(np.float64) == tie, tf, np.float32(0))
    # keep pairs normalised after rounding lo to float
    bad = np.abs(lo.astype(np.float64)) > 0.5 * ulp
    lo[bad] = 0.0
    want = hi.astype(np.float64) + lo.astype(np.float64)
    th, tl = torch.from_numpy(hi).to(cuda), torch.from_numpy(lo).to(cuda)
    out = torch.empty(n, dtype=torch.float64, device=cuda)
    _lib.check(_lib.lib().tridi_selfcheck_df_to_double(th.data_ptr(), tl.data_ptr(), out.data_ptr(), n,
                                                       ctypes.c_void_p(0)), "selfcheck")
    got = out.cpu().numpy()
    mism = np.flatnonzero(got != want)
    assert mism.size == 0, f"{mism.size} mismatches, first hi={hi[mism[0]]!r} lo={lo[mism[0]]!r}"
