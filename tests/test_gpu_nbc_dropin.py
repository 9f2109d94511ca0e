"""GPU parity of the bank-conflict-free shared-memory CR (crNBC / crNBC32 /
crpcrNBC) and of the host-pointer drop-in launchers.  Tolerances:
tests/parity.py."""
import numpy as np
import pytest

import tridiagonalsolvers_gb300 as tg
from oracle import gold
from tridiagonalsolvers_gb300 import dropin, workloads

from .parity import check_against_oracle, check_ulps, check_ulps_where_reference_valid, legacy_accept

pytestmark = pytest.mark.gpu
NP = {"f32": np.float32, "f64": np.float64}


def _dev(cuda, *arrs):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(v)).to(cuda) for v in arrs]


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [2, 4, 8, 32, 64, 128, 256, 512, 1024, 2048])
def test_cr_nbc_vs_oracle(cuda, n, prec):
    import torch

    dt = NP[prec]
    for m in (1, 5, 77):
        a, b, c, d = workloads.dominant(m, n, seed=300 + n + m, dtype=dt)
        t = _dev(cuda, a, b, c, d)
        x = tg.crNBC(*t).cpu().numpy()
        x32 = tg.crNBC32(*t).cpu().numpy()
        assert tg.device_status() == 0
        check_against_oracle(a, b, c, d, x, dtype=dt)
        assert np.array_equal(x, x32)
        # the same CR arithmetic as the register kernel: agreement to a few ulp
        xr = tg.cr(*t).cpu().numpy()
        check_ulps(x, xr, ulps=4)


TUNE_NBC_KERNEL = 8  # tridi.h: TRIDI_TUNE_NBC_KERNEL (2 = the shared-memory kernel)


@pytest.fixture
def shared_memory_kernel():
    from tridiagonalsolvers_gb300 import _lib

    L = _lib.lib()
    _lib.check(L.tridi_set_tunable(TUNE_NBC_KERNEL, 2), "tridi_set_tunable")
    yield
    L.tridi_set_tunable(TUNE_NBC_KERNEL, 0)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [2, 4, 32, 64, 256, 1024, 2048])
def test_shared_memory_kernel_matches_register_cr(cuda, shared_memory_kernel, n, prec):
    """The shared-memory CR (compacted levels, register tail) against the FP64
    oracle, and bit for bit against the register CR: the same arithmetic."""
    dt = NP[prec]
    for m in (1, 33):
        a, b, c, d = workloads.dominant(m, n, seed=500 + n + m, dtype=dt)
        t = _dev(cuda, a, b, c, d)
        x = tg.crNBC(*t).cpu().numpy()
        assert tg.device_status() == 0
        check_against_oracle(a, b, c, d, x, dtype=dt)
        assert np.array_equal(x, tg.cr(*t).cpu().numpy())


@pytest.mark.parametrize("n", [8, 64, 256])
def test_shared_memory_crpcr_sweep(cuda, shared_memory_kernel, n):
    a, b, c, d = workloads.dominant(19, n, seed=27 + n)
    t = _dev(cuda, a, b, c, d)
    rest = 2
    while rest <= n // 2:
        x = tg.crpcrNBC(*t, rest).cpu().numpy()
        check_against_oracle(a, b, c, d, x)
        check_ulps(x, tg.crpcr(*t, rest_system_size=rest).cpu().numpy())
        rest *= 2


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [8, 64, 256, 1024])
def test_crpcr_nbc_sweep(cuda, n, prec):
    dt = NP[prec]
    a, b, c, d = workloads.dominant(19, n, seed=17 + n, dtype=dt)
    t = _dev(cuda, a, b, c, d)
    rest = 2
    while rest <= n // 2:
        x = tg.crpcrNBC(*t, rest).cpu().numpy()
        check_against_oracle(a, b, c, d, x, dtype=dt)
        rest *= 2


def test_nbc_misaligned_direct_path(cuda):
    import torch

    n, m = 128, 9
    a, b, c, d = workloads.dominant(m, n, seed=8)
    bufs = [torch.zeros(m * n + 1, dtype=torch.float32, device=cuda) for _ in range(5)]
    views = [t_[1:] for t_ in bufs]
    for v, h in zip(views[:4], (a, b, c, d)):
        v.copy_(torch.from_numpy(h.ravel()))
    tg.crNBC(*views[:4], x=views[4], system_size=n)
    check_against_oracle(a, b, c, d, views[4].view(m, n).cpu().numpy())


def _ref():
    if not gold.RefKernels.available():
        pytest.skip("reference kernels not built")
    return gold.RefKernels()


@pytest.mark.parametrize("kind", ["crNBC", "crNBC32"])
@pytest.mark.parametrize("n", [16, 64, 256, 1024])
def test_nbc_vs_reference_kernel(cuda, kind, n):
    import torch

    rk = _ref()
    a, b, c, d = workloads.dominant(48, n, seed=61 + n)
    t = _dev(cuda, a, b, c, d)
    xr = torch.zeros_like(t[0])
    rk.solve(kind, *t, xr, n, 48, 0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    a2, b2, c2, d2 = _dev(cuda, a, b, c, d)
    x = tg.crNBC(a2, b2, c2, d2).cpu().numpy()
    check_ulps_where_reference_valid(x, xr.cpu().numpy(), a, b, c, d)


@pytest.mark.parametrize("n", [64, 256])
def test_crpcr_nbc_vs_reference_kernel(cuda, n):
    import torch

    rk = _ref()
    a, b, c, d = workloads.dominant(24, n, seed=71 + n)
    rest = 2
    while rest <= n // 2:
        t = _dev(cuda, a, b, c, d)
        xr = torch.zeros_like(t[0])
        rk.solve("crpcrNBC", *t, xr, n, 24, rest, torch.cuda.current_stream().cuda_stream)
        x = tg.crpcrNBC(*_dev(cuda, a, b, c, d), rest).cpu().numpy()
        check_ulps(x, xr.cpu().numpy())
        rest *= 2


# ---- host-pointer drop-ins ---------------------------------------------------
@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("name", ["cr", "pcr", "crNBC", "crNBC32"])
def test_dropin_matches_device_path(cuda, name, prec):
    dt = NP[prec]
    n, m = 256, 3000  # several chunks of whole systems
    a, b, c, d = workloads.dominant(m, n, seed=5, dtype=dt)
    keep = [v.copy() for v in (a, b, c, d)]
    x = np.zeros_like(a)
    getattr(dropin, name)(a, b, c, d, x, n, m)
    for u, v in zip((a, b, c, d), keep):
        assert np.array_equal(u, v)
    dev_fn = {"cr": tg.cr, "pcr": tg.pcr, "crNBC": tg.crNBC, "crNBC32": tg.crNBC32}[name]
    xd = dev_fn(*_dev(cuda, a, b, c, d)).cpu().numpy()
    from tridiagonalsolvers_gb300._lib import lib

    if name == "pcr" and prec == "f32" and lib().tridi_dropin_pageable_in_place():
        # solved in place from the pageable arrays: the hybrid kernel's PCR (plain
        # loads) against the two-phase PCR kernel of the device path
        check_ulps(x, xd, ulps=64)
    else:
        assert np.array_equal(x, xd)
    check_against_oracle(a, b, c, d, x, dtype=dt)
    if prec == "f32":
        legacy_accept(x, a, b, c, d)


@pytest.mark.parametrize("name", ["crpcr", "crpcrNBC"])
def test_dropin_hybrids(cuda, name):
    n, m = 512, 700
    a, b, c, d = workloads.dominant(m, n, seed=6)
    for rest in (2, 16, 256):
        x = np.zeros_like(a)
        getattr(dropin, name)(a, b, c, d, x, n, m, rest)
        check_against_oracle(a, b, c, d, x)


def test_dropin_large_batch_chunks(cuda):
    n, m = 256, 65536
    a, b, c, d = workloads.dominant(m, n, seed=workloads.SEEDS["c2"])
    x = np.zeros_like(a)
    dropin.cr(a, b, c, d, x, n, m)
    sel = np.r_[0:32, 8190:8194, m - 32:m]
    check_against_oracle(a[sel], b[sel], c[sel], d[sel], x[sel])


def test_dropin_rejects_bad_sizes(cuda):
    a = np.zeros((2, 300), np.float32)
    with pytest.raises(tg.TridiError):
        dropin.cr(a, a.copy(), a.copy(), a.copy(), a.copy(), 300, 2)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [256, 1024])
def test_dropin_pinned_arrays_solved_in_place(cuda, prec, n):
    """Pinned, mapped host arrays (torch's pin_memory): the launchers solve them
    in place over the host link (TRIDI_TUNE_DROPIN_MAPPED, key 11); the same
    calls staged through device memory (key 11 = 2) agree -- bit for bit where
    both paths run the same CR arithmetic -- and a..d are left unchanged."""
    import torch

    from tridiagonalsolvers_gb300._lib import lib

    dt = NP[prec]
    m = 300
    a, b, c, d = workloads.dominant(m, n, seed=77 + n, dtype=dt)

    def pinned(v):
        return torch.from_numpy(np.ascontiguousarray(v).reshape(-1).copy()).pin_memory().numpy()

    pa, pb, pc, pd = (pinned(v) for v in (a, b, c, d))
    launchers = [("cr", dropin.cr, ()), ("pcr", dropin.pcr, ()), ("crpcr", dropin.crpcr, (32,)),
                 ("crNBC", dropin.crNBC, ()), ("crNBC32", dropin.crNBC32, ()),
                 ("crpcrNBC", dropin.crpcrNBC, (32,))]
    L = lib()
    for name, fn, extra in launchers:
        x_in = pinned(np.zeros(m * n, dt))
        fn(pa, pb, pc, pd, x_in, n, m, *extra)
        x_st = pinned(np.zeros(m * n, dt))
        assert L.tridi_set_tunable(11, 2) == 0
        try:
            fn(pa, pb, pc, pd, x_st, n, m, *extra)
        finally:
            L.tridi_set_tunable(11, 0)
        check_against_oracle(a, b, c, d, x_in.reshape(m, n), dtype=dt)
        check_against_oracle(a, b, c, d, x_st.reshape(m, n), dtype=dt)
        # staged, pcr and crpcr at 1024 unknowns take the two-phase / register PCR kernels;
        # in place, the hybrid kernel's (plain loads): the same algorithm, other rounding
        if name == "pcr" or (prec == "f32" and n == 1024 and name in ("crpcr", "crpcrNBC")):
            check_ulps(x_in.reshape(m, n), x_st.reshape(m, n), ulps=64)
        else:
            assert np.array_equal(x_in, x_st), name
    for p, v in zip((pa, pb, pc, pd), (a, b, c, d)):
        assert np.array_equal(p, np.ascontiguousarray(v).reshape(-1))
    assert tg.device_status() == 0


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("n", [64, 256, 1024])
def test_dropin_pageable_arrays_solved_in_place(cuda, n, prec):
    """The host-pointer launchers on ordinary (pageable) numpy arrays: where
    the device reaches pageable memory through the host's page tables
    (tridi_dropin_pageable_in_place() = 1, as on Grace hosts) the solver works
    on them in place; the same calls with pageable arrays staged
    (TRIDI_TUNE_DROPIN_MAPPED = 3) and fully staged (= 2) agree -- bit for
    bit where both paths run the same CR arithmetic -- and a..d are left
    unchanged."""
    from tridiagonalsolvers_gb300._lib import lib

    L = lib()
    print("pageable in place:", L.tridi_dropin_pageable_in_place())
    dt = NP[prec]
    m = 301
    a, b, c, d = workloads.dominant(m, n, seed=91 + n, dtype=dt)
    pa, pb, pc, pd = (np.ascontiguousarray(v).reshape(-1).copy() for v in (a, b, c, d))
    launchers = [("cr", dropin.cr, ()), ("pcr", dropin.pcr, ()), ("crpcr", dropin.crpcr, (16,)),
                 ("crNBC", dropin.crNBC, ()), ("crNBC32", dropin.crNBC32, ()),
                 ("crpcrNBC", dropin.crpcrNBC, (16,))]
    for name, fn, extra in launchers:
        x_in = np.ones(m * n, dt)
        fn(pa, pb, pc, pd, x_in, n, m, *extra)
        check_against_oracle(a, b, c, d, x_in.reshape(m, n), dtype=dt)
        for mode in (3, 2):
            x_st = np.ones(m * n, dt)
            assert L.tridi_set_tunable(11, mode) == 0
            try:
                fn(pa, pb, pc, pd, x_st, n, m, *extra)
            finally:
                L.tridi_set_tunable(11, 0)
            check_against_oracle(a, b, c, d, x_st.reshape(m, n), dtype=dt)
            # staged, pcr and crpcr at 1024 unknowns take the two-phase / register PCR kernels;
            # in place, the hybrid kernel's PCR (plain loads): the same algorithm, other rounding
            if name == "pcr" or (prec == "f32" and n == 1024 and name in ("crpcr", "crpcrNBC")):
                check_ulps(x_in.reshape(m, n), x_st.reshape(m, n), ulps=64)
            else:
                assert np.array_equal(x_in, x_st), (name, mode)
    for p, v in zip((pa, pb, pc, pd), (a, b, c, d)):
        assert np.array_equal(p, np.ascontiguousarray(v).reshape(-1))
    assert tg.device_status() == 0


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_dropin_pageable_every_launcher_and_size(cuda, prec):
    """Every host-pointer launcher at every power-of-two size its kernels
    take, on pageable arrays: the in-place path (where the device reaches
    pageable memory) returns the staged path's status and its answer passes
    the FP64 oracle, within a few ulp of the staged answer."""
    from tridiagonalsolvers_gb300._lib import lib

    L = lib()
    dt = NP[prec]
    f = L.tridi_dropin_solve_f32 if prec == "f32" else L.tridi_dropin_solve_f64
    nmax = 4096 if prec == "f32" else 2048
    m = 3
    for algo, name in enumerate(["cr", "pcr", "crpcr", "crNBC", "crpcrNBC", "crNBC32"]):
        n = 2
        while n <= nmax:
            a, b, c, d = (np.ascontiguousarray(v).reshape(-1) for v in workloads.dominant(m, n, seed=n, dtype=dt))
            param = max(2, n // 4) if name in ("crpcr", "crpcrNBC") else 0
            x_in, x_st = np.ones(m * n, dt), np.ones(m * n, dt)
            s_in = f(algo, *(v.ctypes.data for v in (a, b, c, d, x_in)), n, m, param)
            assert L.tridi_set_tunable(11, 3) == 0
            try:
                s_st = f(algo, *(v.ctypes.data for v in (a, b, c, d, x_st)), n, m, param)
            finally:
                L.tridi_set_tunable(11, 0)
            assert s_in == s_st, (name, n, L.tridi_status_string(s_in), L.tridi_status_string(s_st))
            if s_in == 0:
                check_against_oracle(a.reshape(m, n), b.reshape(m, n), c.reshape(m, n), d.reshape(m, n),
                                     x_in.reshape(m, n), dtype=dt)
                check_ulps(x_in.reshape(m, n), x_st.reshape(m, n), ulps=64)
            n *= 2
    assert tg.device_status() == 0


@pytest.mark.parametrize("n", [2, 8, 32, 64, 512, 2048, 4096])
def test_dropin_pinned_cr_sizes(cuda, n):
    """cr() on pinned, mapped arrays across the system sizes (warp and block
    shapes of the hybrid kernels reading host memory directly), against the
    staged path bit for bit and against the FP64 oracle."""
    import torch

    from tridiagonalsolvers_gb300._lib import lib

    m = 33
    a, b, c, d = workloads.dominant(m, n, seed=5 + n)

    def pinned(v):
        return torch.from_numpy(np.ascontiguousarray(v).reshape(-1).copy()).pin_memory().numpy()

    pa, pb, pc, pd = (pinned(v) for v in (a, b, c, d))
    x_in = pinned(np.zeros(m * n, np.float32))
    dropin.cr(pa, pb, pc, pd, x_in, n, m)
    x_st = pinned(np.zeros(m * n, np.float32))
    L = lib()
    assert L.tridi_set_tunable(11, 2) == 0
    try:
        dropin.cr(pa, pb, pc, pd, x_st, n, m)
    finally:
        L.tridi_set_tunable(11, 0)
    check_against_oracle(a, b, c, d, x_in.reshape(m, n))
    assert np.array_equal(x_in, x_st)
