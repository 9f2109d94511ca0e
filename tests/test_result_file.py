"""The reference-format result dump (tridi_write_result_file_*) is byte for
byte the reference's writeResultToFile (tridiagonal_gold.h:96-107), compiled
from the reference sources into oracle/_ref when they are present, else
checked against the format's definition."""
import numpy as np
import pytest

from oracle import gold
from tridiagonalsolvers_gb300.dropin import write_result_file


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_dump_matches_reference_writer(tmp_path, dtype):
    rng = np.random.default_rng(7)
    m, n = 3, 5
    x = (rng.standard_normal(m * n) * 10.0 ** rng.integers(-8, 8, m * n)).astype(dtype)
    x[0], x[1], x[2] = 0.0, -0.0, 1.0 / 3.0
    ours = tmp_path / "ours.txt"
    write_result_file(x, m, n, ours)
    text = ours.read_text()
    lines = text.splitlines()
    assert len(lines) == m * (n + 1)
    for s in range(m):
        assert lines[s * (n + 1)] == f"***The following is the result of the equation set {s}"
        for i in range(n):
            assert float(lines[s * (n + 1) + 1 + i]) == pytest.approx(float(x[s * n + i]), rel=1e-5, abs=0)
    suf = "f32" if dtype == np.float32 else "f64"
    ref = gold.ref_gold_lib(suf)
    if ref is None:
        pytest.skip("reference build not present")
    theirs = tmp_path / "ref.txt"
    xr = x.copy()
    getattr(ref, f"ref_write_result_file_{suf}")(xr.ctypes.data_as(__import__("ctypes").c_void_p), m, n,
                                                   str(theirs).encode())
    assert theirs.read_bytes() == ours.read_bytes()
