"""Loader of the native library (libtridi.so, built by build.py) and ctypes
signatures of its C ABI (include/tridi.h).

There is no CPU fallback: if the library is missing or was built for another
machine, loading raises, and every solver call fails loudly.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_size_t, c_uint, c_void_p
from pathlib import Path

from . import build as _build

_LIB: ctypes.CDLL | None = None


class TridiError(RuntimeError):
    """A C-ABI call returned a status other than TRIDI_SUCCESS."""

    def __init__(self, status: int, what: str):
        self.status = status
        lib = _LIB
        msg = lib.tridi_status_string(status).decode() if lib else str(status)
        extra = ""
        if lib and status == 4:
            extra = f" (cudaError {lib.tridi_last_cuda_error()})"
        super().__init__(f"{what}: {msg}{extra} [status {status}]")


# name -> (restype, argtypes)
_P = c_void_p
_SIGS: dict[str, tuple] = {
    "tridi_version": (c_char_p, []),
    "tridi_status_string": (c_char_p, [c_int]),
    "tridi_last_cuda_error": (c_int, []),
    "tridi_init": (c_int, []),
    "tridi_device_status": (c_int, [POINTER(c_uint), c_int]),
    "tridi_set_tunable": (c_int, [c_int, c_int]),
    "tridi_get_tunable": (c_int, [c_int]),
}
for _prec in ("f32", "f64"):
    for _name in ("cr", "pcr", "cr_nbc"):
        _SIGS[f"tridi_{_name}_{_prec}"] = (c_int, [_P, _P, _P, _P, _P, c_int, c_int, _P])
    for _name in ("crpcr", "crpcr_nbc"):
        _SIGS[f"tridi_{_name}_{_prec}"] = (c_int, [_P, _P, _P, _P, _P, c_int, c_int, c_int, _P])
    _SIGS[f"tridi_solve_{_prec}"] = (c_int, [_P, _P, _P, _P, _P, c_int, c_int, _P])
    _SIGS[f"tridi_pcr_thomas_{_prec}"] = (c_int, [_P, _P, _P, _P, _P, c_int, c_int, c_int, _P])
    _SIGS[f"tridi_dropin_solve_{_prec}"] = (c_int, [c_int, _P, _P, _P, _P, _P, c_int, c_int, c_int])
    _SIGS[f"tridi_solve_large_{_prec}"] = (c_int, [_P, _P, _P, _P, _P, ctypes.c_long, ctypes.c_long, c_int, _P,
                                                   c_size_t, _P])
_SIGS["tridi_dropin_release"] = (c_int, [])
_SIGS["tridi_dropin_pageable_in_place"] = (c_int, [])
_SIGS["tridi_write_result_file_f32"] = (c_int, [_P, c_int, c_int, c_char_p])
_SIGS["tridi_write_result_file_f64"] = (c_int, [_P, c_int, c_int, c_char_p])
_SIGS["tridi_large_workspace_bytes"] = (c_size_t, [ctypes.c_long, ctypes.c_long, c_int])
_SIGS["tridi_ragged_plan_create"] = (c_int, [_P, c_int, POINTER(c_void_p)])
_SIGS["tridi_ragged_plan_create_refine"] = (c_int, [_P, c_int, POINTER(c_void_p)])
_SIGS["tridi_ragged_plan_device_bytes"] = (c_size_t, [_P])
_SIGS["tridi_ragged_plan_items"] = (c_int, [_P])
_SIGS["tridi_ragged_plan_upload"] = (c_int, [_P, _P, c_size_t, _P])
_SIGS["tridi_ragged_plan_destroy"] = (c_int, [_P])
_SIGS["tridi_ragged_solve_f32"] = (c_int, [_P, _P, _P, _P, _P, _P, _P, _P])
_SIGS["tridi_ragged_plan_total_rows"] = (ctypes.c_long, [_P])
_SIGS["tridi_ragged_plan_num_systems"] = (c_int, [_P])
_SIGS["tridi_ragged_refine_workspace_bytes"] = (c_size_t, [ctypes.c_long, ctypes.c_long])
_SIGS["tridi_ragged_refine_f32"] = (c_int, [_P, _P, _P, _P, _P, _P, _P, _P, c_int, _P, c_size_t, _P, _P])
_SIGS["tridi_noalloc_max_unknowns"] = (ctypes.c_long, [])
_SIGS["tridi_noalloc_last_cuda_error"] = (c_int, [])
_SIGS["tridi_solve_interleaved_noalloc_f32"] = (c_int, [_P, _P, _P, _P, _P, ctypes.c_long, ctypes.c_long, _P])
_LL = ctypes.c_longlong
_SIGS["tridi_selfcheck_wait"] = (c_int, [ctypes.c_longlong, c_int, _P, c_int, _P])
_SIGS["tridi_selfcheck_df_to_double"] = (c_int, [_P, _P, _P, ctypes.c_long, _P])
_SIGS["tridi_autotune"] = (c_int, [c_int, ctypes.c_long, ctypes.c_long, _P, POINTER(c_int),
                                   POINTER(ctypes.c_float)])
_SIGS["tridi_tuned"] = (c_int, [c_int, ctypes.c_long])
_SIGS["tridi_set_tuned"] = (c_int, [c_int, ctypes.c_long, c_int])
_SIGS["tridi_autotune_reset"] = (c_int, [])
_SIGS["tridi_server_create"] = (c_int, [c_size_t, ctypes.c_long, c_int, c_int, c_int, POINTER(c_void_p)])
_SIGS["tridi_server_request_footprint"] = (c_size_t, [ctypes.c_long, ctypes.c_long])
_SIGS["tridi_server_submit"] = (c_int, [_P, _P, _P, _P, _P, _P, _P, c_int, c_double, POINTER(_LL)])
_SIGS["tridi_server_wait"] = (c_int, [_P, _LL, c_int, POINTER(c_int), POINTER(c_int), POINTER(c_double),
                                      POINTER(c_double)])
_SIGS["tridi_server_stats"] = (c_int, [_P, POINTER(_LL), POINTER(_LL), POINTER(_LL), POINTER(c_double)])
_SIGS["tridi_server_phase_times"] = (c_int, [_P, POINTER(c_double), c_int])
_SIGS["tridi_server_destroy"] = (c_int, [_P])
_SIGS["tridi_refine_workspace_bytes"] = (c_size_t, [ctypes.c_long, ctypes.c_long, c_int])
_SIGS["tridi_refine_f32"] = (c_int, [_P, _P, _P, _P, _P, ctypes.c_long, ctypes.c_long, c_int, c_double, c_int, _P,
                                     c_size_t, _P, POINTER(c_int), POINTER(c_double)])


def declared_symbols() -> list[str]:
    """Every function the public headers declare (parsed from include/*.h)."""
    import re

    names: list[str] = []
    for h in sorted((_build.INCLUDE).glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        if "extern \"C\"" not in text:
            continue
        for mt in re.finditer(r"\b(tridi_[a-z0-9_]+)\s*\(", text):
            if mt.group(1) not in names:
                names.append(mt.group(1))
    return names


def lib(build_if_missing: bool = False) -> ctypes.CDLL:
    """The loaded library.  Raises if it is missing (unless asked to build)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = Path(_build.LIB)
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(
                f"{path} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')"
            )
        _build.build()
    dll = ctypes.CDLL(str(path))
    for name, (res, args) in _SIGS.items():
        fn = getattr(dll, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _LIB = dll
    return dll


def check(status: int, what: str) -> None:
    if status != 0:
        raise TridiError(status, what)
