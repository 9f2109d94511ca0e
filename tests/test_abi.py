"""The C ABI library loads and exports every function include/*.h declares
(no GPU needed: nothing here launches work)."""
import ctypes

from tridiagonalsolvers_gb300 import _lib


def test_every_declared_symbol_is_exported(native):
    names = _lib.declared_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(native, n)]
    assert not missing, f"declared in include/*.h but not exported: {missing}"


def test_status_strings_and_version(native):
    assert b"sm_103a" in native.tridi_version()
    for s in range(10):
        assert native.tridi_status_string(s)
    assert native.tridi_status_string(0) == b"success"


def test_argument_validation_needs_no_gpu(native):
    # Null pointers and bad sizes are rejected before any CUDA call.
    null = ctypes.c_void_p(0)
    assert native.tridi_cr_f32(null, null, null, null, null, 256, 4, null) == 1
    p = ctypes.c_void_p(256)
    assert native.tridi_cr_f32(p, p, p, p, p, 0, 4, null) == 2
    assert native.tridi_cr_f32(p, p, p, p, p, 256, 0, null) == 1
    assert native.tridi_cr_f32(p, p, p, p, p, 300, 4, null) == 2
    assert native.tridi_crpcr_f32(p, p, p, p, p, 256, 4, 3, null) == 2
    assert native.tridi_crpcr_f32(p, p, p, p, p, 256, 4, 256, null) == 2
    assert native.tridi_pcr_f32(p, p, p, p, p, 8192, 4, null) == 2


def test_pageable_query_answers_without_a_gpu(native):
    # 1 only where a device reaches pageable memory through the host's page
    # tables; with no usable device the answer is 0, not an error.
    v = native.tridi_dropin_pageable_in_place()
    assert v in (0, 1)
    import torch

    if not torch.cuda.is_available():
        assert v == 0
