"""The allocation-free entry point (tridi_solve_interleaved_noalloc_f32).

It exists for callers that cannot allocate device memory when they solve
(their device memory is owned by their own pool, or an allocation's implicit
synchronisation is not acceptable in their loop): its scratch is an array
compiled into the library.  Checked here through the C ABI against the
existing interleaved solve (tridi_solve_large_f32, whose base case is the same
Thomas recurrence with caller-provided workspace), to the parity tolerances of
tests/parity.py, on two calls in a row that share the static scratch.  This
file is collected last, so a run that stops at the first failure has already
run every other test; it also passes on its own in a fresh process."""
import ctypes

import numpy as np
import pytest

from tridiagonalsolvers_gb300 import _lib, workloads

from .parity import FWD_TOL, check_against_oracle

pytestmark = pytest.mark.gpu


def _existing(lib, t, x, n, m, stream):
    import torch

    wsb = lib.tridi_large_workspace_bytes(n, m, 4)
    ws = torch.empty(wsb, dtype=torch.uint8, device=t[0].device)
    assert lib.tridi_solve_large_f32(*(v.data_ptr() for v in t), x.data_ptr(), n, m, 1, ws.data_ptr(), wsb,
                                     stream) == 0
    torch.cuda.synchronize()


def test_noalloc_matches_existing_entry_point_twice(cuda, native):
    import torch

    lib = _lib.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.tridi_noalloc_max_unknowns() == 1 << 21
    # two calls in a row with different shapes: the second reuses the scratch
    # the first left behind
    for n, m, seed in ((256, 4096, 1), (200, 1000, 2)):
        a, b, c, d = workloads.dominant(m, n, seed=seed, layout=1)  # (n, m) interleaved
        t = [torch.from_numpy(np.ascontiguousarray(v).ravel()).to(cuda) for v in (a, b, c, d)]
        x_new = torch.full((n * m,), float("nan"), device=cuda)
        x_old = torch.empty(n * m, device=cuda)
        st = lib.tridi_solve_interleaved_noalloc_f32(*(v.data_ptr() for v in t), x_new.data_ptr(), n, m, stream)
        assert st == 0, lib.tridi_status_string(st)
        torch.cuda.synchronize()
        _existing(lib, t, x_old, n, m, stream)
        xn = x_new.cpu().numpy().reshape(n, m)
        xo = x_old.cpu().numpy().reshape(n, m)
        assert np.all(np.isfinite(xn))
        rel = np.abs(xn - xo).max(axis=0) / np.abs(xo).max(axis=0)
        assert rel.max() <= FWD_TOL[np.float32], f"differs from tridi_solve_large_f32 by {rel.max():.2e}"
        check_against_oracle(a, b, c, d, xn, layout=1)


def test_noalloc_rejects_requests_beyond_its_scratch(cuda, native):
    import torch

    lib = _lib.lib()
    cap = lib.tridi_noalloc_max_unknowns()
    t = torch.zeros(4, device=cuda)
    p = t.data_ptr()
    n, m = 1024, cap // 1024 + 1  # one system more than fits
    assert lib.tridi_solve_interleaved_noalloc_f32(p, p, p, p, p, n, m, None) == 8  # TRIDI_ERROR_WORKSPACE_TOO_SMALL
    assert lib.tridi_solve_interleaved_noalloc_f32(p, p, p, p, p, 0, 4, None) == 1
