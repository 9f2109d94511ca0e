"""Parity on every benchmark configuration at its full stated shape, with
EVERY system checked against the FP64 oracle (no sampling):

  512 x 512 plain FP32 (seed 1001): cr, pcr, crNBC, crNBC32, pcrGauss, and
      crpcr / crpcrNBC at every switch level; also the reference's own
      kernels rebuilt for sm_103a (64 ulp where their answer solves the system)
  65536 x 256 and 16384 x 1024 (seeds 1002, 1012): the same solvers, the
      whole hybrid switch-level sweep, and the host-pointer drop-in
  1024 x 65536 interleaved, weakly dominant (seed 1003): plain FP32 and
      refined to 1e-10 in both residual arithmetics
  100000 ragged ADI systems, sizes log-uniform in [32, 8192] (seed 1004):
      plain and refined to 1e-10 in both residual arithmetics

Tolerances: tests/parity.py (FP32: residual 2e-6, forward error 2e-5; weakly
dominant FP32: 1e-5 / 5e-3; refined: residual 1e-10)."""
import numpy as np
import pytest

import tridiagonalsolvers_gb300 as tg
from oracle import gold
from tridiagonalsolvers_gb300 import dropin, workloads
from tridiagonalsolvers_gb300.ragged import RaggedPlan, RaggedRefiner, padded

from .parity import RES_TOL, check_against_oracle, check_ulps_where_reference_valid, legacy_accept

pytestmark = pytest.mark.gpu
WEAK = dict(res_tol=1e-5, fwd_tol=5e-3)
REFINED_TOL = 1e-10


def _dev(cuda, *arrs):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(v)).to(cuda) for v in arrs]


def _solvers(n):
    """(name, call) for every uniform-size solver at system size n."""
    out = [("cr", lambda t: tg.cr(*t)), ("pcr", lambda t: tg.pcr(*t)), ("crNBC", lambda t: tg.crNBC(*t)),
           ("crNBC32", lambda t: tg.crNBC32(*t)), ("pcrGauss", lambda t: tg.pcrGauss(*t, 0))]
    rest = 2
    while rest <= n // 2:
        out.append((f"crpcr{rest}", lambda t, r=rest: tg.crpcr(*t, r)))
        out.append((f"crpcrNBC{rest}", lambda t, r=rest: tg.crpcrNBC(*t, r)))
        rest *= 2
    return out


def _all_solvers_full(cuda, m, n, seed):
    a, b, c, d = workloads.dominant(m, n, seed=seed)
    x64 = gold.solve_f64(a, b, c, d)
    t = _dev(cuda, a, b, c, d)
    worst = {}
    for name, fn in _solvers(n):
        x = fn(t).cpu().numpy()
        assert tg.device_status() == 0, name
        try:
            worst[name] = check_against_oracle(a, b, c, d, x, x64=x64)
        except AssertionError as e:
            raise AssertionError(f"{name} at {m} x {n}: {e}") from None
    print({k: f"{v[0]:.1e}/{v[1]:.1e}" for k, v in worst.items()})
    return a, b, c, d, x64


def test_c1_512x512_every_solver_every_system(cuda):
    m, n = 512, 512
    a, b, c, d, _ = _all_solvers_full(cuda, m, n, workloads.SEEDS["c1"])
    x = tg.cr(*_dev(cuda, a, b, c, d)).cpu().numpy()
    legacy_accept(x, a, b, c, d)


def test_c1_512x512_against_reference_kernels(cuda):
    import torch

    if not gold.RefKernels.available():
        pytest.skip("reference kernels not built")
    rk = gold.RefKernels()
    m, n = 512, 512
    a, b, c, d = workloads.dominant(m, n, seed=workloads.SEEDS["c1"])
    cases = [("cr", 0, lambda t: tg.cr(*t)), ("pcr", 0, lambda t: tg.pcr(*t)),
             ("crNBC", 0, lambda t: tg.crNBC(*t)), ("crNBC32", 0, lambda t: tg.crNBC32(*t))]
    rest = 2
    while rest <= n // 2:
        cases.append(("crpcr", rest, lambda t, r=rest: tg.crpcr(*t, r)))
        cases.append(("crpcrNBC", rest, lambda t, r=rest: tg.crpcrNBC(*t, r)))
        rest *= 2
    for kind, rest, fn in cases:
        t = _dev(cuda, a, b, c, d)
        xr = torch.zeros_like(t[0])
        rk.solve(kind, *t, xr, n, m, rest, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        x = fn(_dev(cuda, a, b, c, d)).cpu().numpy()
        compared, ref_wrong = check_ulps_where_reference_valid(x, xr.cpu().numpy(), a, b, c, d)
        assert compared + ref_wrong == m
        print(f"{kind} rest={rest}: {compared} systems within 64 ulp of the reference kernel, "
              f"{ref_wrong} where the reference kernel's answer fails the oracle")


def test_c2_65536x256_every_solver_every_system(cuda):
    m, n = 65536, 256
    a, b, c, d, x64 = _all_solvers_full(cuda, m, n, workloads.SEEDS["c2"])
    # the host-pointer drop-in on the whole batch (pipelined chunks)
    x = np.zeros_like(a)
    dropin.cr(a, b, c, d, x, n, m)
    check_against_oracle(a, b, c, d, x, x64=x64)
    legacy_accept(x, a, b, c, d)


def test_c2_16384x1024_every_solver_every_system(cuda):
    _all_solvers_full(cuda, 16384, 1024, workloads.SEEDS["c2b"])


def test_c3_1024x65536_interleaved_plain_every_system(cuda):
    n, m = 65536, 1024
    a, b, c, d = workloads.weak(m, n, seed=workloads.SEEDS["c3"], layout=1)
    x = tg.solve_large(*(v.ravel() for v in _dev(cuda, a, b, c, d)), n, m, "interleaved")
    assert tg.device_status() == 0
    x = x.cpu().numpy().reshape(n, m)
    # checked system by system in the contiguous layout (the oracle's fast path)
    at, bt, ct, dt_, xt = (np.ascontiguousarray(v.T) for v in (a, b, c, d, x))
    check_against_oracle(at, bt, ct, dt_, xt, **WEAK)


@pytest.mark.parametrize("residual", ["df", "fp64"])
def test_c3_1024x65536_refined_every_system(cuda, residual):
    import torch

    n, m = 65536, 1024
    a, b, c, d = workloads.weak(m, n, seed=workloads.SEEDS["c3"], layout=1)
    x, sweeps, rel = tg.refine(*(v.ravel() for v in _dev(cuda, a, b, c, d)), n, m, layout="interleaved",
                               tol=REFINED_TOL, max_sweeps=20, residual=residual)
    assert bool(torch.isfinite(x).all())
    at, bt, ct, dt_, xt = (np.ascontiguousarray(v.T) for v in (a, b, c, d, x.cpu().numpy().reshape(n, m)))
    res = gold.rel_residual(at, bt, ct, dt_, xt)
    assert res.max() <= REFINED_TOL, f"oracle residual {res.max():.2e} (kernel said {rel:.2e}) after {sweeps} sweeps"
    x64 = gold.solve_f64(at, bt, ct, dt_)
    fwd = (np.abs(xt - x64).max(axis=1) / np.abs(x64).max(axis=1)).max()
    assert fwd < 1e-7, f"forward error {fwd:.2e}"
    # the kernel's own maximum agrees with the oracle's
    assert rel <= 4 * res.max() + 1e-13 and res.max() <= 4 * rel + 1e-13
    print(f"1024x65536 refined ({residual}): {sweeps} sweeps, residual {res.max():.2e}, fwd {fwd:.2e}")


def _c4():
    sizes = workloads.ragged_sizes(100000, 32, 8192, seed=workloads.SEEDS["c4"])
    a, b, c, d, off = workloads.adi(sizes, seed=workloads.SEEDS["c4"])
    return a, b, c, d, off


def _ragged_dev(cuda, v, total):
    import torch

    t = torch.zeros(padded(total), dtype=torch.float32, device=cuda)
    t[:total] = torch.from_numpy(v)
    return t


def test_c4_ragged_100000_plain_every_system(cuda):
    a, b, c, d, off = _c4()
    total = int(off[-1])
    x = RaggedPlan(off).solve(*(_ragged_dev(cuda, v, total) for v in (a, b, c, d))).cpu().numpy()[:total]
    assert tg.device_status() == 0
    res, fwd = gold.check_ragged(a, b, c, d, x, off)
    assert res.max() <= RES_TOL[np.float32], f"system {res.argmax()}: residual {res.max():.2e}"
    assert fwd.max() <= 2e-5, f"system {fwd.argmax()}: forward error {fwd.max():.2e}"


@pytest.mark.parametrize("residual", ["df", "fp64"])
def test_c4_ragged_100000_refined_every_system(cuda, residual):
    a, b, c, d, off = _c4()
    total = int(off[-1])
    t = [_ragged_dev(cuda, v, total) for v in (a, b, c, d)]
    plan = RaggedPlan(off, refine=True)
    x, rel = RaggedRefiner(plan, *t, sweeps=1, graph=False, residual=residual).run()
    assert tg.device_status() == 0
    x = x.cpu().numpy()[:total]
    res, fwd = gold.check_ragged(a, b, c, d, x, off)
    assert res.max() <= REFINED_TOL, f"system {res.argmax()}: residual {res.max():.2e}"
    assert fwd.max() <= 1e-9, f"system {fwd.argmax()}: forward error {fwd.max():.2e}"
    assert rel <= 2 * res.max() + 1e-15 and res.max() <= 2 * rel + 1e-15
    print(f"ragged 100000 refined ({residual}): residual {res.max():.2e}, fwd {fwd.max():.2e}")
