"""GPU parity of PCR-then-Thomas (tridi_pcr_thomas_*, the device work behind
pcrGaussWrapper, pcrGauss_app.cu:164).  Tolerances: tests/parity.py."""
from pathlib import Path

import numpy as np
import pytest

import tridiagonalsolvers_gb300 as tg
from oracle import gold
from tridiagonalsolvers_gb300 import dropin, workloads

from .parity import check_against_oracle, check_ulps, check_ulps_where_reference_valid, legacy_accept

pytestmark = pytest.mark.gpu
NP = {"f32": np.float32, "f64": np.float64}
GOLDEN = Path(__file__).parent / "golden" / "reference_gold.npz"


def _dev(cuda, *arrs):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(v)).to(cuda) for v in arrs]


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [1, 2, 8, 64, 100, 256, 1000, 1024, 2048, 4096])
def test_pcr_thomas_every_g(cuda, n, prec):
    dt = NP[prec]
    a, b, c, d = workloads.dominant(9, n, seed=900 + n, dtype=dt)
    t = _dev(cuda, a, b, c, d)
    g = 1
    while g <= n:
        x = tg.pcrGauss(*t, g).cpu().numpy()
        check_against_oracle(a, b, c, d, x, dtype=dt)
        g *= 4 if n > 256 else 2
    assert tg.device_status() == 0


def test_pcr_thomas_weak_systems_exact_for_large_g(cuda):
    # the reference's g=64 table entry (3 PCR steps) is only approximate; with
    # log2(g) steps the result is exact also on weakly dominant systems
    a, b, c, d = workloads.weak(16, 1024, seed=4)
    x = tg.pcrGauss(*_dev(cuda, a, b, c, d), 64).cpu().numpy()
    check_against_oracle(a, b, c, d, x, res_tol=1e-5, fwd_tol=5e-3)


@pytest.mark.parametrize("n", [16, 256, 1024])
@pytest.mark.parametrize("g", [1, 2, 4, 8])
def test_pcr_thomas_vs_reference_kernel(cuda, n, g):
    """pcrGaussSmall with g in {1,2,4,8}: the reference's table gives log2(g)
    PCR steps there (pcrGauss_app.cu:61-72), so its result is exact too."""
    import torch

    if not gold.RefKernels.available():
        pytest.skip("reference kernels not built")
    rk = gold.RefKernels()
    m = 24
    a, b, c, d = workloads.dominant(m, n, seed=3 + n + g)
    ta, tb, tc, td = _dev(cuda, a, b, c, d)
    a2, b2, c2, d2 = (torch.zeros_like(ta) for _ in range(4))
    second = rk.pcr_gauss(ta, tb, tc, td, a2, b2, c2, d2, n, m, g, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    xr = (d2 if second else td).cpu().numpy()
    x = tg.pcrGauss(*_dev(cuda, a, b, c, d), g).cpu().numpy()
    check_against_oracle(a, b, c, d, x)
    check_ulps_where_reference_valid(x, xr, a, b, c, d)


def test_reference_driver_configuration(cuda):
    """test_tridiagonal.cpp:30-31,81,107: 2 x 8192 from testGeneration (srand
    default), pcrGaussWrapper(..., 64), RMS <= 1e-3 against the gold solver.
    Here also checked against the reference gold's own output (golden file)."""
    n, m = 8192, 2
    a, b, c, d = gold.generate_reference_inputs(n, m, np.float32, seed=1)
    x = np.zeros_like(a)
    dropin.pcrGaussWrapper(a, b, c, d, x, n, m, 64)
    legacy_accept(x, a, b, c, d)
    check_against_oracle(a, b, c, d, x)
    x_gold = np.load(GOLDEN)["n8192_m2_s1_f32_x"]
    assert np.sqrt(np.mean((x - x_gold) ** 2, axis=1)).max() < 1e-6


def test_reference_large_pcr_gauss_path_is_approximate(cuda):
    """The reference's own large path (globalPCROneBlockSystem + chunked
    pcrKernelBranchFree) on the driver configuration: it passes the
    reference's 1e-3 acceptance but is not exact; ours is."""
    import torch

    if not gold.RefKernels.available():
        pytest.skip("reference kernels not built")
    rk = gold.RefKernels()
    n, m = 8192, 2
    a, b, c, d = gold.generate_reference_inputs(n, m, np.float32, seed=1)
    ta, tb, tc, td = _dev(cuda, a, b, c, d)
    a2, b2, c2, d2 = (torch.zeros_like(ta) for _ in range(4))
    second = rk.pcr_gauss(ta, tb, tc, td, a2, b2, c2, d2, n, m, 64, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    xr = (d2 if second else td).cpu().numpy()
    legacy_accept(xr, a, b, c, d)
    x = np.zeros_like(a)
    dropin.pcrGaussWrapper(a, b, c, d, x, n, m, 64)
    res_ref = gold.rel_residual(a, b, c, d, xr).max()
    res_new = gold.rel_residual(a, b, c, d, x).max()
    assert res_new <= max(res_ref, 2e-6)


# pcrGaussWrapper at every size the reference's large path accepts: the
# reference takes any systemSize > MINSYSTEM = 1024 down its global-memory PCR
# path (pcrGauss_app.cu:196-228, :102-162); its driver calls it at 2 x 8192
# (test_tridiagonal.cpp:30-31,81).  Here: PCR-then-Thomas up to 4096 rows, the
# partition solver up to 8704 (FP32) / 4608 (FP64) rows, the large-system
# solver beyond, through the host-pointer drop-in.
@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n,m", [(8192, 2), (16384, 4), (65536, 2), (10007, 3), (5000, 3), (80000, 1)])
def test_pcr_gauss_wrapper_large_sizes(cuda, prec, n, m):
    dt = NP[prec]
    if n == 8192:
        a, b, c, d = gold.generate_reference_inputs(n, m, dt, seed=1)
    else:
        a, b, c, d = workloads.dominant(m, n, seed=40 + n + m, dtype=dt)
    keep = [v.copy() for v in (a, b, c, d)]
    x = np.zeros_like(a)
    dropin.pcrGaussWrapper(a, b, c, d, x, n, m, 64)
    for u, v in zip((a, b, c, d), keep):
        assert np.array_equal(u, v)
    check_against_oracle(a, b, c, d, x, dtype=dt)
    legacy_accept(x, a, b, c, d)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_pcr_gauss_wrapper_large_weakly_dominant(cuda, prec):
    dt = NP[prec]
    n, m = 32768, 3
    a, b, c, d = workloads.weak(m, n, seed=12, dtype=dt)
    x = np.zeros_like(a)
    dropin.pcrGaussWrapper(a, b, c, d, x, n, m, 64)
    if prec == "f32":
        check_against_oracle(a, b, c, d, x, res_tol=1e-5, fwd_tol=5e-3)
    else:
        check_against_oracle(a, b, c, d, x, dtype=dt, res_tol=1e-13, fwd_tol=1e-10)


def test_pcr_gauss_wrapper_large_many_chunks(cuda):
    """Enough 16384-row systems for several pipelined chunks sharing one
    scratch slice of the large solver's workspace."""
    n, m = 16384, 300
    a, b, c, d = workloads.dominant(m, n, seed=77)
    x = np.zeros_like(a)
    dropin.pcrGaussWrapper(a, b, c, d, x, n, m, 64)
    check_against_oracle(a, b, c, d, x)


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024])
def test_pcr_thomas_register_kernel_every_split(cuda, n):
    """The register PCR-then-Thomas kernel (FP32, 64..1024 unknowns, g < n/2)
    for every split, including partial warp tiles (m not a multiple of the
    systems a warp tile holds) and one system: against the FP64 oracle, and
    within a few ulp of the shared-memory kernel (TRIDI_TUNE_PCR_KERNEL = 2)."""
    from tridiagonalsolvers_gb300._lib import lib

    L = lib()
    for m in (1, 7, 130):
        a, b, c, d = workloads.dominant(m, n, seed=11 * n + m)
        t = _dev(cuda, a, b, c, d)
        g = 1
        while g < n // 2:
            x = tg.pcrGauss(*t, g).cpu().numpy()
            check_against_oracle(a, b, c, d, x)
            assert L.tridi_set_tunable(10, 2) == 0
            try:
                xs = tg.pcrGauss(*t, g).cpu().numpy()
            finally:
                L.tridi_set_tunable(10, 0)
            check_ulps(x, xs, ulps=16)
            g *= 2
    assert tg.device_status() == 0
