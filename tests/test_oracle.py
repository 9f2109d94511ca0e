"""The oracle is pinned before it is trusted: the CPU restatement (oracle/gold.c)
must reproduce the reference's own gold routines bit for bit, both the
reference compiled here (oracle/_ref, skipped where the reference tree is
absent) and the committed golden vectors made from it (tests/golden)."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

from oracle import gold

GOLDEN = Path(__file__).parent / "golden" / "reference_gold.npz"
CASES = [(8192, 2, 1), (512, 4, 7), (64, 5, 11), (2, 3, 3)]
DTYPES = [(np.float32, "f32"), (np.float64, "f64")]


@pytest.mark.parametrize("n,m,seed", CASES)
@pytest.mark.parametrize("dt,tag", DTYPES)
def test_port_matches_golden_vectors(n, m, seed, dt, tag):
    g = np.load(GOLDEN)
    key = f"n{n}_m{m}_s{seed}_{tag}"
    a, b, c, d = gold.generate_reference_inputs(n, m, dt, seed=seed)
    h = hashlib.sha256(b"".join(np.ascontiguousarray(v).tobytes() for v in (a, b, c, d))).digest()
    assert h == g[f"{key}_inputs_sha256"].tobytes(), "port of testGeneration differs from the reference's"
    x = gold.serial_many(a, b, c, d)
    assert np.array_equal(x, g[f"{key}_x"]), "port of the gold Thomas solver differs from the reference's"


def _ref_built():
    return gold.ref_gold_lib("f32") is not None


@pytest.mark.skipif(not _ref_built(), reason="reference tree absent: oracle/_ref not built here")
@pytest.mark.parametrize("dt,tag", DTYPES)
@pytest.mark.parametrize("n,m", [(1024, 3), (256, 8), (4, 9), (3000, 2)])
def test_port_matches_reference_build(dt, tag, n, m):
    a, b, c, d = gold.generate_reference_inputs(n, m, dt, seed=5, use_ref=True)
    a2, b2, c2, d2 = gold.generate_reference_inputs(n, m, dt, seed=5)
    for u, v in zip((a, b, c, d), (a2, b2, c2, d2)):
        assert np.array_equal(u, v)
    assert np.array_equal(gold.serial_many(a, b, c, d), gold.serial_many(a, b, c, d, use_ref=True))
    assert np.array_equal(gold.multithread_many(a, b, c, d), gold.multithread_many(a, b, c, d, use_ref=True))


@pytest.mark.skipif(not _ref_built(), reason="reference tree absent: oracle/_ref not built here")
def test_port_matches_reference_on_seeded_dominant_inputs():
    from tridiagonalsolvers_gb300 import workloads

    a, b, c, d = workloads.dominant(64, 512, seed=3)
    assert np.array_equal(gold.serial_many(a, b, c, d), gold.serial_many(a, b, c, d, use_ref=True))


def test_multithread_skips_remainder_like_the_reference():
    # tridiagonal_gold.h:59,65-67: chunk = m/4, the m % 4 trailing systems are never solved.
    a, b, c, d = gold.generate_reference_inputs(16, 6, np.float32, seed=2)
    x = gold.multithread_many(a, b, c, d)
    ref = gold.serial_many(a, b, c, d)
    assert np.array_equal(x[:4], ref[:4])
    assert np.all(x[4:] == 0)


def test_serial_does_not_touch_callers_arrays():
    a, b, c, d = gold.generate_reference_inputs(32, 2, np.float32, seed=4)
    keep = [v.copy() for v in (a, b, c, d)]
    gold.serial_many(a, b, c, d)
    for u, v in zip((a, b, c, d), keep):
        assert np.array_equal(u, v)


def test_hand_checkable_systems():
    # identity, pure diagonal and a 2x2 with a known solution
    n = 8
    a = np.zeros((1, n), np.float64); c = np.zeros((1, n), np.float64)
    b = np.full((1, n), 2.0); d = np.arange(n, dtype=np.float64)[None]
    assert np.allclose(gold.serial_many(a, b, c, d), d / 2)
    a2 = np.array([[0.0, 1.0]]); b2 = np.array([[2.0, 3.0]]); c2 = np.array([[1.0, 0.0]]); d2 = np.array([[3.0, 4.0]])
    assert np.allclose(gold.serial_many(a2, b2, c2, d2), [[1.0, 1.0]])


def test_fp64_oracle_and_residual():
    from tridiagonalsolvers_gb300 import workloads

    a, b, c, d = workloads.dominant(16, 256, seed=9)
    x = gold.solve_f64(a, b, c, d)
    assert gold.rel_residual(a, b, c, d, x).max() < 1e-14
    x32 = gold.serial_many(a, b, c, d)
    r32 = gold.rel_residual(a, b, c, d, x32)
    assert 1e-9 < r32.max() < 1e-5
    # interleaved layout gives the same solution
    ai, bi, ci, di = (np.ascontiguousarray(v.T) for v in (a, b, c, d))
    xi = gold.solve_f64(ai, bi, ci, di, layout=1)
    assert np.array_equal(xi.T, x)
    assert gold.rel_residual(ai, bi, ci, di, xi, layout=1).max() < 1e-14


def test_compare_many_counts_failures_and_nan():
    x1 = np.zeros((3, 4), np.float32)
    x2 = x1.copy()
    x2[1, 0] = 1.0
    x2[2, 0] = np.nan
    nf, rms = gold.compare_many(x1, x2, 1e-3)
    assert nf == 2
    assert rms[0] == 0 and abs(rms[1] - 0.5) < 1e-7


def test_ragged_check_matches_uniform_routines():
    """gold_check_ragged on a batch of equal sizes gives the uniform routines'
    residuals, and zero forward error for the oracle's own FP64 solution."""
    from tridiagonalsolvers_gb300 import workloads

    m, n = 37, 129
    a, b, c, d = workloads.dominant(m, n, seed=5)
    off = np.arange(m + 1, dtype=np.int64) * n
    x64 = gold.solve_f64(a, b, c, d)
    res, fwd = gold.check_ragged(a.ravel(), b.ravel(), c.ravel(), d.ravel(), x64.ravel(), off)
    assert np.array_equal(res, gold.rel_residual(a, b, c, d, x64))
    assert np.all(fwd == 0)
    x32 = x64.astype(np.float32)
    res, fwd = gold.check_ragged(a.ravel(), b.ravel(), c.ravel(), d.ravel(), x32.ravel(), off)
    assert np.array_equal(res, gold.rel_residual(a, b, c, d, x32))
    assert np.allclose(fwd, np.abs(x32 - x64).max(axis=1) / np.abs(x64).max(axis=1), rtol=0, atol=0)
