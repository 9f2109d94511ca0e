"""GPU parity of the any-size partition solver (tridi_solve_*) against the FP64
oracle: sizes that are not powers of two, tiny and large systems, one warp
and one CTA per system.  Tolerances: tests/parity.py."""
import numpy as np
import pytest

import tridiagonalsolvers_gb300 as tg
from tridiagonalsolvers_gb300 import workloads

from .parity import check_against_oracle, legacy_accept

pytestmark = pytest.mark.gpu
NP = {"f32": np.float32, "f64": np.float64}
SIZES = [1, 2, 3, 5, 31, 32, 33, 100, 255, 256, 257, 480, 481, 500, 992, 993, 1024, 1500, 2048, 3000, 4096,
         4608, 5000, 8192, 8704]


def _dev(cuda, *arrs):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(v)).to(cuda) for v in arrs]


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", SIZES)
def test_partition_vs_oracle(cuda, n, prec):
    dt = NP[prec]
    if prec == "f64" and n > 4608:
        pytest.skip("FP64 partition solver covers n <= 4608")
    for m in (1, 6, 41):
        a, b, c, d = workloads.dominant(m, n, seed=500 + n + m, dtype=dt)
        x = tg.solve(*_dev(cuda, a, b, c, d), system_size=n).cpu().numpy().reshape(m, n)
        assert tg.device_status() == 0
        check_against_oracle(a, b, c, d, x, dtype=dt)
        if prec == "f32":
            legacy_accept(x, a, b, c, d)


@pytest.mark.parametrize("n", [256, 1024])
def test_partition_weakly_dominant(cuda, n):
    a, b, c, d = workloads.weak(64, n, seed=77)
    x = tg.solve(*_dev(cuda, a, b, c, d)).cpu().numpy()
    check_against_oracle(a, b, c, d, x, res_tol=1e-5, fwd_tol=5e-3)


def test_partition_adi_lines(cuda):
    sizes = np.full(50, 700)
    a, b, c, d, off = workloads.adi(sizes, seed=3)
    shp = (50, 700)
    x = tg.solve(*_dev(cuda, *(v.reshape(shp) for v in (a, b, c, d)))).cpu().numpy()
    check_against_oracle(*(v.reshape(shp) for v in (a, b, c, d)), x)


def test_partition_ignores_a0_and_c_last(cuda):
    # like the gold solver, a[0] and c[n-1] are treated as zero
    n, m = 300, 4
    a, b, c, d = workloads.dominant(m, n, seed=1)
    a2, c2 = a.copy(), c.copy()
    a2[:, 0] = 0.7
    c2[:, -1] = -0.3
    x1 = tg.solve(*_dev(cuda, a, b, c, d)).cpu().numpy()
    x2 = tg.solve(*_dev(cuda, a2, b, c2, d)).cpu().numpy()
    assert np.array_equal(x1, x2)


def test_partition_large_batch(cuda):
    m, n = 65536, 256
    a, b, c, d = workloads.dominant(m, n, seed=workloads.SEEDS["c2"])
    x = tg.solve(*_dev(cuda, a, b, c, d)).cpu().numpy()
    sel = np.r_[0:64, m - 64:m]
    check_against_oracle(a[sel], b[sel], c[sel], d[sel], x[sel])
    assert np.all(np.isfinite(x))
