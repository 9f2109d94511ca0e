"""The bounded device waits' timeout path, exercised without faulting or
hanging the GPU: a self-check kernel waits on an mbarrier that nothing
arrives at (no bulk copy is issued into it) with a short limit, and must
return with TRIDI_DEVERR_WAIT_TIMEOUT set in the device status word, which
tridi_device_status() reports and then clears."""
import ctypes

import numpy as np
import pytest

import tridiagonalsolvers_gb300 as tg
from tridiagonalsolvers_gb300 import _lib, workloads

from .parity import check_against_oracle

pytestmark = pytest.mark.gpu
WAIT_TIMEOUT = 0x1  # TRIDI_DEVERR_WAIT_TIMEOUT
LIMIT = 20000       # SM cycles, ~10 us


def _status(reset):
    bits = ctypes.c_uint(0)
    _lib.check(_lib.lib().tridi_device_status(ctypes.byref(bits), reset), "tridi_device_status")
    return bits.value


def _selfcheck(cuda, arrive, threads=64, limit=LIMIT):
    import torch

    flags = torch.full((threads,), -1, dtype=torch.int32, device=cuda)
    _lib.check(_lib.lib().tridi_selfcheck_wait(limit, arrive, flags.data_ptr(), threads, ctypes.c_void_p(0)),
               "tridi_selfcheck_wait")
    torch.cuda.synchronize()
    return flags.cpu().numpy()


def test_completed_wait_sets_nothing(cuda):
    _status(reset=1)
    flags = _selfcheck(cuda, arrive=1)
    assert np.all(flags == 0)
    assert _status(reset=0) == 0


def test_wait_that_runs_out_is_reported_and_cleared(cuda):
    _status(reset=1)
    flags = _selfcheck(cuda, arrive=0, threads=96)
    assert np.all(flags == 1), "every thread's wait must run out and return"
    assert _status(reset=1) & WAIT_TIMEOUT
    assert _status(reset=0) == 0, "tridi_device_status(reset=1) must clear the bit"
    assert tg.device_status() == 0
    # the context stays usable: a solve afterwards is correct and clean
    a, b, c, d = workloads.dominant(8, 256, seed=3)
    import torch

    x = tg.cr(*(torch.from_numpy(v).to(cuda) for v in (a, b, c, d))).cpu().numpy()
    check_against_oracle(a, b, c, d, x)
    assert _status(reset=0) == 0


def test_selfcheck_rejects_bad_arguments(cuda):
    L = _lib.lib()
    null = ctypes.c_void_p(0)
    assert L.tridi_selfcheck_wait(LIMIT, 0, null, 32, null) == 1
    p = ctypes.c_void_p(256)
    assert L.tridi_selfcheck_wait(LIMIT, 0, p, 0, null) == 1
    assert L.tridi_selfcheck_wait(LIMIT, 0, p, 2048, null) == 1
    assert L.tridi_selfcheck_wait(0, 0, p, 32, null) == 1
    assert L.tridi_selfcheck_wait(10 ** 12, 0, p, 32, null) == 1
