"""The reference's C++ launchers themselves, called from a C++ program
(tests/cpp/dropin_caller.cpp) that declares them as the reference's driver
does (test_tridiagonal.cpp:17-26), in float and in double: results equal the
Python drop-in's bit for bit and pass the FP64 oracle; the reference's timing
line (cr_app.cu:40-48, numIterations = 50) behind TRIDI_DROPIN_TIMING=1; the
print-and-exit error behaviour of CUDA_SAFE_CALL, and TRIDI_DROPIN_NO_EXIT=1.
Tolerances: tests/parity.py."""
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import gold
from tridiagonalsolvers_gb300 import dropin, workloads

from . import cpp_caller
from .parity import check_against_oracle, legacy_accept

pytestmark = pytest.mark.gpu
NP = {"f32": np.float32, "f64": np.float64}
GOLDEN = Path(__file__).parent / "golden" / "reference_gold.npz"
LAUNCHERS = [("cr", 0), ("pcr", 0), ("crpcr", 16), ("crNBC", 0), ("crpcrNBC", 16), ("crNBC32", 0),
             ("pcrGaussWrapper", 64)]


def _py_dropin(launcher, a, b, c, d, n, m, param):
    x = np.zeros_like(a)
    fn = getattr(dropin, launcher)
    if launcher in ("crpcr", "crpcrNBC", "pcrGaussWrapper"):
        fn(a, b, c, d, x, n, m, param)
    else:
        fn(a, b, c, d, x, n, m)
    return x


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("launcher,param", LAUNCHERS)
def test_cpp_launcher(cuda, tmp_path, prec, launcher, param):
    dt = NP[prec]
    n, m = 256, 300
    a, b, c, d = workloads.dominant(m, n, seed=2024, dtype=dt)
    p, x = cpp_caller.run(prec, launcher, a, b, c, d, n, m, param, tmp_path)
    assert p.returncode == 0, p.stdout + p.stderr
    assert p.stdout.strip() == "returned"  # no timing line unless asked for
    assert np.array_equal(x, _py_dropin(launcher, a, b, c, d, n, m, param))
    check_against_oracle(a, b, c, d, x, dtype=dt)
    legacy_accept(x, a, b, c, d)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_cpp_reference_driver_case(cuda, tmp_path, prec):
    """test_tridiagonal.cpp's own call: testGeneration inputs, 2 x 8192,
    pcrGaussWrapper(..., 64), then gpu_result.txt in the reference's format and
    the 1e-3 RMS acceptance against the gold solver (:103-107).  In the
    USE_DOUBLE build this call used to end in exit(1)."""
    dt = NP[prec]
    n, m = 8192, 2
    a, b, c, d = gold.generate_reference_inputs(n, m, dt, seed=1)
    p, x = cpp_caller.run(prec, "pcrGaussWrapper", a, b, c, d, n, m, 64, tmp_path, result_txt=True)
    assert p.returncode == 0, p.stdout + p.stderr
    check_against_oracle(a, b, c, d, x, dtype=dt)
    legacy_accept(x, a, b, c, d)
    txt = (tmp_path / "gpu_result_pcrGaussWrapper.txt").read_text().splitlines()
    assert len(txt) == m * (n + 1)
    assert txt[0] == "***The following is the result of the equation set 0"
    vals = np.array([float(v) for i, v in enumerate(txt) if i % (n + 1)]).reshape(m, n)
    x_gold = gold.serial_many(a, b, c, d)
    assert np.sqrt(np.mean((vals - x_gold) ** 2, axis=1)).max() < 1e-3
    if prec == "f32":
        xg = np.load(GOLDEN)["n8192_m2_s1_f32_x"]
        assert np.sqrt(np.mean((x - xg) ** 2, axis=1)).max() < 1e-6


TIMING = re.compile(r"^(\w+): numSystems: (\d+), systemSize: (\d+), GPU kernel time: ([0-9.]+) ms$")


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_cpp_timing_line(cuda, tmp_path, prec):
    dt = NP[prec]
    n, m = 256, 300
    a, b, c, d = workloads.dominant(m, n, seed=9, dtype=dt)
    env = {"TRIDI_DROPIN_TIMING": "1"}
    p, x = cpp_caller.run(prec, "cr", a, b, c, d, n, m, 0, tmp_path, env=env)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = p.stdout.strip().splitlines()
    assert lines[-1] == "returned" and len(lines) == 2, p.stdout
    mt = TIMING.match(lines[0])
    assert mt and mt.group(1) == "cr" and int(mt.group(2)) == m and int(mt.group(3)) == n, lines[0]
    assert float(mt.group(4)) > 0
    assert np.array_equal(x, _py_dropin("cr", a, b, c, d, n, m, 0))
    # pcrGaussWrapper's line, on the large-system path (its workspace sized for the whole batch)
    n2, m2 = 16384, 40
    a, b, c, d = workloads.dominant(m2, n2, seed=10, dtype=dt)
    p, x = cpp_caller.run(prec, "pcrGaussWrapper", a, b, c, d, n2, m2, 64, tmp_path, env=env)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = p.stdout.strip().splitlines()
    assert re.match(r"^pcrGauss: GPU kernel time: [0-9.]+ ms$", lines[0]), lines[0]
    check_against_oracle(a, b, c, d, x, dtype=dt)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_cpp_error_exits_like_cuda_safe_call(cuda, tmp_path, prec):
    """An unsupported size (cr needs a power of two) is rejected on the host
    before any launch: the launcher prints the error and exits with status 1,
    or, with TRIDI_DROPIN_NO_EXIT=1, prints it and returns."""
    dt = NP[prec]
    n, m = 300, 2
    a, b, c, d = workloads.dominant(m, n, seed=1, dtype=dt)
    p, _ = cpp_caller.run(prec, "cr", a, b, c, d, n, m, 0, tmp_path)
    assert p.returncode == 1
    assert "returned" not in p.stdout
    assert "cr(systemSize=300, numSystems=2) failed: unsupported system size" in p.stderr
    p, _ = cpp_caller.run(prec, "cr", a, b, c, d, n, m, 0, tmp_path, env={"TRIDI_DROPIN_NO_EXIT": "1"})
    assert p.returncode == 0
    assert p.stdout.strip() == "returned"
    assert "failed: unsupported system size" in p.stderr
