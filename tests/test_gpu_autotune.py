"""Autotuner on the GPU: every decision is taken from a timed candidate, lands
in the table, is used by what comes next (plans, pcr_thomas with gaussian = 0,
refinement) and leaves results correct."""
import numpy as np
import pytest

from oracle import gold
from tridiagonalsolvers_gb300 import autotune, workloads
from tridiagonalsolvers_gb300.ragged import RaggedPlan, padded

from .parity import RES_TOL

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _clean_table():
    autotune.reset()
    yield
    autotune.reset()


def test_tune_ragged_buckets_and_solve(cuda):
    import torch

    for k in (64, 1024, 4096):
        th, ms = autotune.tune("ragged", k, sample_unknowns=1 << 22)
        assert th in (32, 160, 480) and ms > 0
        assert autotune.table()["ragged"][str(1 << (k.bit_length() - 1))] == th
    # force every bucket to each choice in turn: results stay correct
    sizes = np.array([40, 100, 700, 1500, 3000, 5000, 8000, 300, 64])
    a, b, c, d, off = workloads.adi(sizes, seed=4)
    total = int(off[-1])

    def dev(v):
        t = torch.zeros(padded(total), dtype=torch.float32, device=cuda)
        t[:total] = torch.from_numpy(v)
        return t

    for th in (32, 160, 480):
        autotune.set_table({"ragged": {str(1 << k): th for k in range(5, 15)}})
        x = RaggedPlan(off).solve(dev(a), dev(b), dev(c), dev(d)).cpu().numpy()[:total]
        for s in range(len(sizes)):
            lo, hi = off[s], off[s + 1]
            sl = [v[lo:hi][None] for v in (a, b, c, d)]
            assert gold.rel_residual(*sl, x[lo:hi][None])[0] <= RES_TOL[np.float32], (th, s)


@pytest.mark.parametrize("n", [64, 256, 1024])
def test_tune_crpcr_rest(cuda, n):
    rest, ms = autotune.tune("crpcr_rest", n, sample_unknowns=1 << 22)
    assert 2 <= rest <= n // 2 and rest & (rest - 1) == 0 and ms > 0
    assert autotune.table()["crpcr_rest"][str(n)] == rest


@pytest.mark.parametrize("n", [32, 256, 1000])
def test_tune_pcr_thomas_split_then_auto(cuda, n):
    import torch

    import tridiagonalsolvers_gb300 as tg

    if n & (n - 1) == 0:
        g, ms = autotune.tune("pcr_thomas", n, sample_unknowns=1 << 22)
        assert 1 <= g <= n and g & (g - 1) == 0 and ms > 0
    a, b, c, d = workloads.dominant(64, n, seed=3)
    t = [torch.from_numpy(v).to(cuda) for v in (a, b, c, d)]
    x = tg.pcrGauss(*t, gaussian=0).cpu().numpy()
    assert gold.rel_residual(a, b, c, d, x).max() <= RES_TOL[np.float32]


def test_table_round_trip(tmp_path, cuda):
    autotune.set_table({"ragged": {"64": 160}, "crpcr_rest": {"256": 16}, "pcr_thomas": {"128": 8}})
    p = tmp_path / "t.json"
    autotune.save(str(p))
    autotune.reset()
    assert autotune.table()["ragged"]["64"] == 0
    autotune.load(str(p))
    t = autotune.table()
    assert t["ragged"]["64"] == 160 and t["crpcr_rest"]["256"] == 16 and t["pcr_thomas"]["128"] == 8


@pytest.mark.parametrize("n", [64, 512, 1024, 2048])
def test_tune_cr_rows_then_solve(cuda, n):
    import torch

    import tridiagonalsolvers_gb300 as tg

    rows, ms = autotune.tune("cr_rows", n, sample_unknowns=1 << 22)
    assert rows in (4, 8, 16) and ms > 0
    assert autotune.table()["cr_rows"][str(n)] == rows
    a, b, c, d = workloads.dominant(96, n, seed=12)
    t = [torch.from_numpy(v).to(cuda) for v in (a, b, c, d)]
    for rr in (4, 8, 16):  # every instantiated shape gives a correct CR and CR-PCR
        if n // rr > 256:
            continue
        autotune.set_table({"cr_rows": {str(n): rr}})
        x = tg.cr(*t).cpu().numpy()
        assert gold.rel_residual(a, b, c, d, x).max() <= RES_TOL[np.float32], rr
        for rest in (4, 32):  # rows left after CR: one per warp, or several per warp
            x = tg.crpcr(*t, rest).cpu().numpy()
            assert gold.rel_residual(a, b, c, d, x).max() <= RES_TOL[np.float32], (rr, rest)


def test_tune_ragged_refine_buckets_and_refine(cuda):
    """The refinement's own table: tuned on the fused refinement, read only by
    refinement plans (plain plans keep the plain table), and every forced
    choice refines every system to 1e-10."""
    import torch

    from tridiagonalsolvers_gb300.ragged import RaggedRefiner

    for k in (256, 4096):
        th, ms = autotune.tune("ragged_refine", k, sample_unknowns=1 << 22)
        assert th in (32, 160, 480) and ms > 0
        assert autotune.table()["ragged_refine"][str(k)] == th
    sizes = np.array([40, 100, 700, 1500, 3000, 5000, 8000, 300, 64])
    a, b, c, d, off = workloads.adi(sizes, seed=6)
    total = int(off[-1])

    def dev(v):
        t = torch.zeros(padded(total), dtype=torch.float32, device=cuda)
        t[:total] = torch.from_numpy(v)
        return t

    t = [dev(v) for v in (a, b, c, d)]
    autotune.set_table({"ragged": {str(1 << k): 32 for k in range(5, 15)}})
    plain_items = RaggedPlan(off).items
    for th in (32, 160, 480):
        autotune.set_table({"ragged_refine": {str(1 << k): th for k in range(5, 15)}})
        assert RaggedPlan(off).items == plain_items  # plain plans ignore the refinement's table
        plan = RaggedPlan(off, refine=True)
        x, rel = RaggedRefiner(plan, *t, sweeps=1, graph=False).run()
        x = x.cpu().numpy()[:total]
        assert rel <= 1e-10, th
        for s in range(len(sizes)):
            lo, hi = off[s], off[s + 1]
            sl = [v[lo:hi][None] for v in (a, b, c, d)]
            assert gold.rel_residual(*sl, x[lo:hi][None])[0] <= 1e-10, (th, s)
