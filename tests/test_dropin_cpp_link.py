"""The reference's C++ boundary links against libtridi.so (no GPU needed).

The reference declares its launchers only as bare C++ prototypes in its driver
(test_tridiagonal.cpp:17-26), in float or, with USE_DOUBLE, double
(common.h:8-12).  A caller declaring all seven that way must link against the
library in both precisions (14 overloads), and so must the reference's own
driver, compiled where it lies when its tree is present (oracle/Makefile
target `driver`)."""
import subprocess
from pathlib import Path

import pytest

from tridiagonalsolvers_gb300 import build as pkg_build

from . import cpp_caller

ROOT = Path(__file__).resolve().parents[1]
LAUNCHERS = ["cr", "pcr", "crpcr", "crNBC", "crpcrNBC", "crNBC32", "pcrGaussWrapper"]


def _undefined(exe: Path) -> str:
    return subprocess.run(["nm", "-C", "-u", str(exe)], capture_output=True, text=True, check=True).stdout


@pytest.mark.parametrize("prec,T", [("f32", "float"), ("f64", "double")])
def test_caller_of_all_seven_launchers_links(native, prec, T):
    exe = cpp_caller.build(prec)
    undef = _undefined(exe)
    for name in LAUNCHERS:
        # every launcher is an unresolved C++ symbol of the caller in this precision ...
        assert f"{name}({T}*, {T}*, {T}*, {T}*, {T}*, int, int" in undef, name
    # ... that the library defines with C++ linkage (the reference's mangled names)
    defined = subprocess.run(["nm", "-D", "-C", "--defined-only", str(pkg_build.LIB)],
                             capture_output=True, text=True, check=True).stdout
    for name in LAUNCHERS:
        assert f" {name}({T}*, {T}*, {T}*, {T}*, {T}*, int, int" in defined, name


def test_reference_driver_links(native):
    """The reference's test_tridiagonal.cpp, built in both precisions against
    libtridi.so (skipped where the reference tree is absent)."""
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "driver"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    if "absent" in r.stdout:
        pytest.skip("reference tree not present")
    for prec, T in (("f32", "float"), ("f64", "double")):
        exe = ROOT / "oracle" / "_ref" / f"test_tridiagonal_{prec}"
        assert exe.exists()
        assert f"pcrGaussWrapper({T}*, {T}*, {T}*, {T}*, {T}*, int, int, int)" in _undefined(exe)
