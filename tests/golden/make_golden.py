"""Generates tests/golden/reference_gold.npz from the reference itself.

Run here, where the reference tree exists: it builds oracle/_ref (the
reference's own tridiagonal_gold.h compiled where it lies, see
oracle/Makefile) and records, for each case, the reference generator's
inputs (testGeneration, tridiagonal_gold.h:81-94, after srand(seed); stored
as a SHA-256 of their bytes) and the reference gold solver's output (serialManySystems, tridiagonal_gold.h:47-53),
in FP32 (T = float) and FP64 (-DUSE_DOUBLE).

The first case is the reference driver's own configuration: 2 systems of
8192 unknowns (test_tridiagonal.cpp:30-31), unseeded rand() (= seed 1).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import gold  # noqa: E402

CASES = [  # (n, m, seed)
    (8192, 2, 1),
    (512, 4, 7),
    (64, 5, 11),
    (2, 3, 3),
]


def main() -> None:
    gold.build(ref=True)
    if gold.ref_gold_lib("f32") is None:
        raise SystemExit("oracle/_ref was not built: the reference tree is required")
    out = {}
    for n, m, seed in CASES:
        for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
            a, b, c, d = gold.generate_reference_inputs(n, m, dt, seed=seed, use_ref=True)
            x = gold.serial_many(a, b, c, d, use_ref=True)
            key = f"n{n}_m{m}_s{seed}_{tag}"
            # Inputs are stored as a SHA-256 of their bytes (the oracle's port of
            # the generator must reproduce them exactly); outputs in full.
            h = hashlib.sha256(b"".join(np.ascontiguousarray(v).tobytes() for v in (a, b, c, d)))
            out[f"{key}_inputs_sha256"] = np.frombuffer(h.digest(), np.uint8)
            out[f"{key}_x"] = x
    dst = Path(__file__).with_name("reference_gold.npz")
    np.savez_compressed(dst, **out)
    print(f"wrote {dst} ({dst.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
