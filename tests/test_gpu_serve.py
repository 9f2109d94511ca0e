"""GPU tests of the continuous-batching server (tridi_server_*): results reach
the 1e-10 relative residual target against the FP64 oracle, a request's
result is the same alone and in a mix (to 1e-9 relative), admission by HBM
footprint rejects what can never fit and queues what must wait, and batches
overlap on the device."""
import threading

import numpy as np
import pytest

from oracle import gold
from tridiagonalsolvers_gb300 import TridiError
from tridiagonalsolvers_gb300.serve import Server, make_request

pytestmark = pytest.mark.gpu


def _check(req, x, tol=1.5e-10):
    a, b, c, d, off = req
    for s in range(len(off) - 1):
        lo, hi = off[s], off[s + 1]
        res = gold.rel_residual(a[lo:hi][None], b[lo:hi][None], c[lo:hi][None], d[lo:hi][None], x[lo:hi][None])[0]
        assert res <= tol, f"system {s} (n={hi - lo}) residual {res:.2e}"


def test_alone_equals_in_mix(cuda):
    rng = np.random.default_rng(7)
    probe = make_request(rng, max_systems=40)
    others = [make_request(rng, max_systems=300) for _ in range(12)]
    srv = Server(hbm_budget_bytes=4 << 30, max_inflight=3)
    try:
        x_alone, info = srv.wait(srv.submit(*probe))
        _check(probe, x_alone)
        ids = [srv.submit(*r) for r in others[:6]] + [srv.submit(*probe)] + [srv.submit(*r) for r in others[6:]]
        outs = [srv.wait(i) for i in ids]
        x_mix = outs[6][0]
        rel = np.abs(x_mix - x_alone).max() / np.abs(x_alone).max()
        assert rel <= 1e-9, f"alone vs mixed differ by {rel:.2e}"
        for r, (x, inf) in zip(others[:6] + [probe] + others[6:], outs):
            assert inf["rel_residual"] <= 1e-10
        _check(others[0], outs[0][0])
        assert srv.stats()["completed"] == 14
    finally:
        srv.close()


def test_admission_by_footprint_and_overlap(cuda):
    rng = np.random.default_rng(11)
    reqs = [make_request(rng, max_systems=200) for _ in range(16)]
    budget = 2 * max(Server.footprint(int(r[4][-1]), len(r[4]) - 1) for r in reqs)
    srv = Server(hbm_budget_bytes=budget, max_inflight=3)
    try:
        ids = []
        lock = threading.Lock()

        def submitter(part):
            for r in part:
                i = srv.submit(*r)
                with lock:
                    ids.append((i, r))

        th = [threading.Thread(target=submitter, args=(reqs[k::2],)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for i, r in ids:
            x, info = srv.wait(i)
            assert info["rel_residual"] <= 1e-10
        st = srv.stats()
        assert st["completed"] == len(reqs)
        assert st["max_inflight_seen"] >= 2, st  # batches ran concurrently
        # a request whose footprint exceeds the whole budget is refused up front
        big = make_request(np.random.default_rng(1), max_systems=1)
        a = np.zeros(budget // 4, np.float32)
        with pytest.raises(TridiError) as ei:
            srv.submit(a, a, a, a, np.array([0, 10000, 20000, len(a) // 2], np.int64))
        assert ei.value.status in (2, 7)
        del big
    finally:
        srv.close()


def test_large_and_small_requests_in_one_batch(cuda):
    """Requests of 2^18 rows or more take the direct copies, smaller ones the
    pinned staging, in the same batch: every answer reaches the target."""
    from tridiagonalsolvers_gb300 import workloads

    rng = np.random.default_rng(21)
    a, b, c, d, off = workloads.adi(np.full(100, 4000), seed=3)
    big = (a, b, c, d, off)  # 400000 rows
    smalls = [make_request(rng, max_systems=30) for _ in range(5)]
    srv = Server(hbm_budget_bytes=4 << 30, max_inflight=1)
    try:
        reqs = [smalls[0], big] + smalls[1:]
        ids = [srv.submit(*r) for r in reqs]
        for r, i in zip(reqs, ids):
            x, info = srv.wait(i)
            assert info["rel_residual"] <= 1e-10
            _check(r, x)
    finally:
        srv.close()
