"""GPU parity of the CR / PCR / hybrid CR-PCR kernels (C ABI tridi_cr_*,
tridi_pcr_*, tridi_crpcr_*) against the FP64 oracle and the reference's own
kernels rebuilt for sm_103a.  Tolerances: tests/parity.py."""
import numpy as np
import pytest

import tridiagonalsolvers_gb300 as tg
from oracle import gold
from tridiagonalsolvers_gb300 import workloads

from .parity import check_against_oracle, check_ulps, check_ulps_where_reference_valid, legacy_accept

pytestmark = pytest.mark.gpu

SIZES = [2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096]
NP = {"f32": np.float32, "f64": np.float64}


def _dev(cuda, *arrs):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(v)).to(cuda) for v in arrs]


def _solve(algo, cuda, a, b, c, d, rest=None):
    import torch

    ta, tb, tc, td = _dev(cuda, a, b, c, d)
    keep = [t.clone() for t in (ta, tb, tc, td)]
    if algo == "crpcr":
        x = tg.crpcr(ta, tb, tc, td, rest)
    else:
        x = getattr(tg, algo)(ta, tb, tc, td)
    torch.cuda.synchronize()
    assert tg.device_status() == 0
    for u, v in zip((ta, tb, tc, td), keep):
        assert torch.equal(u, v), "inputs were modified"
    return x.cpu().numpy()


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("algo", ["cr", "pcr"])
@pytest.mark.parametrize("n", SIZES)
def test_cr_pcr_vs_oracle(cuda, algo, n, prec):
    dt = NP[prec]
    if prec == "f64" and n > 2048:
        pytest.skip("FP64 CR family covers n <= 2048")
    for m in (1, 7, 133):
        a, b, c, d = workloads.dominant(m, n, seed=100 + n + m, dtype=dt)
        x = _solve(algo, cuda, a, b, c, d)
        check_against_oracle(a, b, c, d, x, dtype=dt)
        if prec == "f32":
            legacy_accept(x, a, b, c, d)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [8, 64, 256, 512, 1024, 2048])
def test_crpcr_switch_level_sweep(cuda, n, prec):
    dt = NP[prec]
    a, b, c, d = workloads.dominant(37, n, seed=7 + n, dtype=dt)
    rest = 2
    while rest <= n // 2:
        x = _solve("crpcr", cuda, a, b, c, d, rest)
        check_against_oracle(a, b, c, d, x, dtype=dt)
        rest *= 2


@pytest.mark.parametrize("n,rest", [(1024, r) for r in (2, 4, 8, 16, 32, 64, 128, 256, 512)]
                         + [(512, r) for r in (2, 4, 16, 64, 256)])
def test_crpcr_register_kernels(cuda, n, rest):
    """The register CR-PCR kernels (FP32, 1024 unknowns: every switch level;
    512 unknowns: batches of 4096 systems and more; rest 2 is cr), on batches
    of one system, a few and more than one wave of warps holds (so warps loop
    over tiles): against the FP64 oracle, and against the shared-memory kernel
    (TRIDI_TUNE_PCR_KERNEL = 2): bit for bit at rest 2 (the same CR
    arithmetic), within a few ulp above (the register kernels' CR levels and
    PCR work on normalised rows)."""
    from tridiagonalsolvers_gb300._lib import lib

    L = lib()
    ms = (1, 5, 2 * 152 * 4 * 2 + 3) if n == 1024 else (4096, 2 * 152 * 8 * 2 + 5)
    for m in ms:
        a, b, c, d = workloads.dominant(m, n, seed=13 * m + rest + n)
        t = _dev(cuda, a, b, c, d)
        x = tg.crpcr(*t, rest).cpu().numpy()
        check_against_oracle(a, b, c, d, x)
        assert L.tridi_set_tunable(10, 2) == 0
        try:
            xs = tg.crpcr(*t, rest).cpu().numpy()
        finally:
            L.tridi_set_tunable(10, 0)
        if rest == 2:
            assert np.array_equal(x, xs)
            assert np.array_equal(x, tg.cr(*t).cpu().numpy())
        else:
            check_ulps(x, xs, ulps=16)
    assert tg.device_status() == 0


def test_reference_driver_case(cuda):
    """The reference driver's inputs (testGeneration, 2 x 8192 after srand(1))
    checked with its own 1e-3 RMS acceptance; CR family limits n to 4096 here,
    so the driver's systems are solved as 4 x 4096 halves of their inputs."""
    a, b, c, d = gold.generate_reference_inputs(4096, 4, np.float32, seed=1)
    x = _solve("cr", cuda, a, b, c, d)
    legacy_accept(x, a, b, c, d)
    check_against_oracle(a, b, c, d, x)


def test_large_batch_65536x256(cuda):
    m, n = 65536, 256
    a, b, c, d = workloads.dominant(m, n, seed=workloads.SEEDS["c2"])
    x = _solve("cr", cuda, a, b, c, d)
    sel = np.r_[0:64, m - 64:m, 4096:4160]
    check_against_oracle(a[sel], b[sel], c[sel], d[sel], x[sel])
    assert np.all(np.isfinite(x))


@pytest.mark.parametrize("n,rest", [(64, None), (1024, None), (1024, 4), (1024, 32), (2048, 64), (1024, 512)])
def test_misaligned_pointers_take_the_direct_path(cuda, n, rest):
    """Inputs 4 bytes off a 16-byte boundary go through the producer-warp
    kernel without bulk copies: warp shapes, and the block shapes' CR levels
    inside warps, gathered intermediate systems and shared-memory PCR."""
    import torch

    m = 10
    a, b, c, d = workloads.dominant(m, n, seed=5 + n)
    bufs = [torch.zeros(m * n + 1, dtype=torch.float32, device=cuda) for _ in range(5)]
    views = [t[1:] for t in bufs]  # 4-byte offset: not 16-byte aligned
    for v, h in zip(views[:4], (a, b, c, d)):
        v.copy_(torch.from_numpy(h.ravel()))
    if rest is None:
        tg.cr(*views[:4], x=views[4], system_size=n)
    else:
        tg.crpcr(*views[:4], rest, x=views[4], system_size=n)
    x = views[4].view(m, n).cpu().numpy()
    check_against_oracle(a, b, c, d, x)
    assert tg.device_status() == 0


# ---- against the reference's own kernels -------------------------------------
def _ref_kernels():
    if not gold.RefKernels.available():
        pytest.skip("reference kernels not built (oracle/_ref/*/ *.cubin absent)")
    return gold.RefKernels()


def _run_ref(rk, kind, cuda, a, b, c, d, rest=0):
    import torch

    ta, tb, tc, td = _dev(cuda, a, b, c, d)
    x = torch.zeros_like(ta)
    m, n = a.shape
    rk.solve(kind, ta, tb, tc, td, x, n, m, rest, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return x.cpu().numpy()


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [4, 16, 64, 256, 512, 1024, 2048])
def test_cr_vs_reference_kernel(cuda, n, prec):
    rk = _ref_kernels()
    dt = NP[prec]
    a, b, c, d = workloads.dominant(64, n, seed=31 + n, dtype=dt)
    xr = _run_ref(rk, "cr", cuda, a, b, c, d)
    x = _solve("cr", cuda, a, b, c, d)
    check_against_oracle(a, b, c, d, x, dtype=dt)
    compared, ref_wrong = check_ulps_where_reference_valid(x, xr, a, b, c, d, dtype=dt)
    if ref_wrong:
        print(f"reference crKernel wrong on {ref_wrong}/{len(a)} systems (n={n}, {prec}): barrier race")


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [4, 16, 64, 256, 512, 1024])
def test_pcr_vs_reference_kernel(cuda, n, prec):
    rk = _ref_kernels()
    dt = NP[prec]
    a, b, c, d = workloads.dominant(64, n, seed=41 + n, dtype=dt)
    xr = _run_ref(rk, "pcr", cuda, a, b, c, d)
    x = _solve("pcr", cuda, a, b, c, d)
    check_against_oracle(a, b, c, d, x, dtype=dt)
    compared, ref_wrong = check_ulps_where_reference_valid(x, xr, a, b, c, d, dtype=dt)
    if ref_wrong:
        print(f"reference pcrKernel wrong on {ref_wrong}/{len(a)} systems (n={n}, {prec})")


@pytest.mark.parametrize("n", [256, 1024])
def test_crpcr_vs_reference_kernel(cuda, n):
    rk = _ref_kernels()
    a, b, c, d = workloads.dominant(32, n, seed=51 + n)
    rest = 2
    while rest <= n // 2:
        if (n + 1) * 5 * 4 + rest * 5 * 4 <= 200 * 1024:
            xr = _run_ref(rk, "crpcr", cuda, a, b, c, d, rest)
            x = _solve("crpcr", cuda, a, b, c, d, rest)
            check_ulps(x, xr)
        rest *= 2
