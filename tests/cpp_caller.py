"""Build and run tests/cpp/dropin_caller.cpp, a C++ caller of the reference's
host launchers declared exactly as the reference's driver declares them
(test_tridiagonal.cpp:17-26), linked against the product's libtridi.so."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

from tridiagonalsolvers_gb300 import build as pkg_build

HERE = Path(__file__).resolve().parent
SRC = HERE / "cpp" / "dropin_caller.cpp"
OUT = HERE / "_build"


def cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand:
            return cand
    raise RuntimeError("no C++ compiler found")


def build(prec: str) -> Path:
    """Compiles the caller for T = float ("f32") or double ("f64", -DUSE_DOUBLE)
    and links it against libtridi.so; raises if it does not link."""
    lib = Path(pkg_build.LIB)
    if not lib.exists():
        pkg_build.build()
    OUT.mkdir(exist_ok=True)
    exe = OUT / f"dropin_caller_{prec}"
    if exe.exists() and exe.stat().st_mtime >= max(SRC.stat().st_mtime, lib.stat().st_mtime):
        return exe
    cmd = [cxx(), "-O2", "-std=c++17", str(SRC), "-o", str(exe), f"-L{lib.parent}", "-ltridi",
           f"-Wl,-rpath,{lib.parent}"]
    if prec == "f64":
        cmd.insert(1, "-DUSE_DOUBLE")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"C++ caller did not build/link:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return exe


def run(prec: str, launcher: str, a, b, c, d, n: int, m: int, param: int, tmp: Path,
        env: dict | None = None, result_txt: bool = False):
    """Runs one launcher through the C++ caller; returns (CompletedProcess, x or None)."""
    dt = np.float32 if prec == "f32" else np.float64
    inp, out = tmp / f"in_{launcher}.bin", tmp / f"out_{launcher}.bin"
    np.concatenate([np.ascontiguousarray(v, dt).ravel() for v in (a, b, c, d)]).tofile(inp)
    if out.exists():
        out.unlink()
    args = [str(build(prec)), launcher, str(n), str(m), str(param), str(inp), str(out)]
    if result_txt:
        args.append(str(tmp / f"gpu_result_{launcher}.txt"))
    full_env = dict(os.environ)
    full_env.update(env or {})
    p = subprocess.run(args, capture_output=True, text=True, env=full_env, timeout=600)
    x = np.fromfile(out, dt).reshape(m, n) if p.returncode == 0 and out.exists() else None
    return p, x
