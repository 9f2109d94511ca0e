"""bench.py's multi-GPU launch path, on CPU: `--gpus N` without a launcher
re-runs the script under torch.distributed.run as N replica ranks (the
reference arm, which needs no GPU, exercises it end to end: rank 0 alone
times the host cores and prints the single JSON line, the other ranks exit 0
without work)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_replica_launch_command():
    argv = bench.replica_launch_argv(["--gpus", "4", "--steps", "3"], 4)
    assert argv[1:4] == ["-m", "torch.distributed.run", "--nnodes=1"]
    assert "--nproc-per-node=4" in argv and "--master-addr=127.0.0.1" in argv
    assert argv[-4:] == ["--gpus", "4", "--steps", "3"]
    assert Path(argv[-5]).name == "bench.py"


def test_world_size_must_match_gpus(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "0")
    with pytest.raises(SystemExit):
        bench.dist_init(4)


def test_two_replica_ranks_print_one_line():
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    env["OMP_NUM_THREADS"] = "2"
    p = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps",
                        "2", "--warmup", "1"], capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["steps"] == 2
    assert rec["value"] > 0 and rec["e2e"]["h2d_bytes_per_step"] == 0
