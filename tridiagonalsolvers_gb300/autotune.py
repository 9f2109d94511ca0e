"""Autotuner front end (the timing and the table are native: tridi_autotune
in csrc/autotune.cu).  Tunes, on the GPU in use:

  * crpcr_rest    -- CR-to-PCR switch level per power-of-two n (4..4096),
                     used by the refinement's FP32 correction solves;
  * pcr_thomas    -- PCR/Thomas split (Thomas chains g) per n (2..4096), used by
                     tridi_pcr_thomas_* with gaussian = 0;
  * ragged        -- threads per system (32, 160, 480) per size bucket
                     [2^k, 2^(k+1)) of the ragged work queue, used by plans
                     created afterwards;
  * cr_rows       -- rows per thread (4, 8, 16) of the FP32 CR / PCR / CR-PCR
                     kernels per power-of-two n (threads per system = n / rows);
  * ragged_refine -- as `ragged`, timed on the fused one-correction refinement,
                     used by plans created afterwards with RaggedPlan(...,
                     refine=True) and by the solve server.

    from tridiagonalsolvers_gb300 import autotune
    table = autotune.tune_all()            # {"ragged": {"32": 32, ...}, ...}
    autotune.save("tuning.json"); autotune.load("tuning.json")
"""
from __future__ import annotations

import ctypes
import json

from ._lib import check, lib

TABLES = {"crpcr_rest": 0, "pcr_thomas": 1, "ragged": 2, "cr_rows": 3, "ragged_refine": 4}
DEFAULT_KEYS = {
    "crpcr_rest": [1 << k for k in range(2, 13)],
    "pcr_thomas": [1 << k for k in range(1, 13)],
    "ragged": [1 << k for k in range(5, 15)],  # buckets [32, 64) .. [16384, 32768)
    "cr_rows": [1 << k for k in range(5, 13)],
    "ragged_refine": [1 << k for k in range(5, 15)],
}


def tune(table: str, key: int, sample_unknowns: int = 1 << 24, stream=None) -> tuple[int, float]:
    """Times the candidates for one key; records and returns (choice, ms)."""
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    chosen, ms = ctypes.c_int(0), ctypes.c_float(0)
    check(lib().tridi_autotune(TABLES[table], int(key), int(sample_unknowns), ctypes.c_void_p(stream.cuda_stream),
                               ctypes.byref(chosen), ctypes.byref(ms)), f"autotune {table} {key}")
    return chosen.value, ms.value


def tune_all(tables=("ragged", "crpcr_rest", "pcr_thomas", "cr_rows", "ragged_refine"),
             sample_unknowns: int = 1 << 24) -> dict:
    out = {}
    for t in tables:
        out[t] = {str(k): tune(t, k, sample_unknowns)[0] for k in DEFAULT_KEYS[t]}
    return out


def table() -> dict:
    L = lib()
    return {t: {str(k): L.tridi_tuned(i, k) for k in DEFAULT_KEYS[t]} for t, i in TABLES.items()}


def set_table(tab: dict) -> None:
    L = lib()
    for t, entries in tab.items():
        for k, v in entries.items():
            check(L.tridi_set_tuned(TABLES[t], int(k), int(v)), f"set_tuned {t} {k}")


def reset() -> None:
    check(lib().tridi_autotune_reset(), "autotune reset")


def save(path: str) -> None:
    with open(path, "w") as f:
        json.dump(table(), f, indent=1, sort_keys=True)


def load(path: str) -> None:
    with open(path) as f:
        set_table(json.load(f))
