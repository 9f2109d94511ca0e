"""Seeded synthetic inputs of the five benchmark workloads.

No public dataset is involved: every workload is a seeded numpy PCG64 draw
with the distribution the benchmark definition states.

  dominant(m, n)   a, c ~ U[-1,1] (a[0] = c[n-1] = 0), b = |a|+|c|+U[1,2],
                   d ~ U[-1,1]: strictly diagonally dominant
                   (512 x 512 plain solve; 65536 x 256 and 16384 x 1024 batches)
  weak(m, n)       same but b = |a|+|c|+U[0.01,0.1]: weakly dominant
                   (1024 x 65536 large-system solve)
  adi(sizes)       a = c = -r, b = 1+2r with r ~ U[0.1,10] per system,
                   d ~ U[-1,1], a[0] = c[n-1] = 0: implicit heat-equation line
                   solves (ragged batch, sizes log-uniform in [32, 8192])
"""
from __future__ import annotations

import numpy as np

# One fixed seed per benchmark workload.
SEEDS = {"c1": 1001, "c2": 1002, "c2b": 1012, "c3": 1003, "c4": 1004, "c5": 1005}


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def dominant(m: int, n: int, seed: int, margin=(1.0, 2.0), dtype=np.float32, layout: int = 0):
    """(a, b, c, d) as (m, n) arrays (layout 0) or (n, m) arrays (layout 1,
    interleaved: element i of system s at i*m + s)."""
    g = _rng(seed)
    shape = (m, n)
    a = g.uniform(-1.0, 1.0, shape)
    c = g.uniform(-1.0, 1.0, shape)
    a[:, 0] = 0.0
    c[:, n - 1] = 0.0
    b = np.abs(a) + np.abs(c) + g.uniform(margin[0], margin[1], shape)
    d = g.uniform(-1.0, 1.0, shape)
    out = tuple(v.astype(dtype) for v in (a, b, c, d))
    if layout == 1:
        out = tuple(np.ascontiguousarray(v.T) for v in out)
    return out


def weak(m: int, n: int, seed: int, dtype=np.float32, layout: int = 0):
    return dominant(m, n, seed, margin=(0.01, 0.1), dtype=dtype, layout=layout)


def ragged_sizes(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """Sizes log-uniform in [lo, hi] (integers, not powers of two)."""
    g = _rng(seed)
    s = np.exp(g.uniform(np.log(lo), np.log(hi + 1), count)).astype(np.int64)
    return np.clip(s, lo, hi)


def adi(sizes: np.ndarray, seed: int, dtype=np.float32):
    """Concatenated ragged ADI systems: returns (a, b, c, d, offsets) with
    offsets[i] the first row of system i (offsets[-1] = total rows)."""
    g = _rng(seed)
    sizes = np.asarray(sizes, np.int64)
    offsets = np.zeros(len(sizes) + 1, np.int64)
    np.cumsum(sizes, out=offsets[1:])
    total = int(offsets[-1])
    r = g.uniform(0.1, 10.0, len(sizes))
    rr = np.repeat(r, sizes)
    a = -rr.copy()
    c = -rr.copy()
    b = 1.0 + 2.0 * rr
    d = g.uniform(-1.0, 1.0, total)
    a[offsets[:-1]] = 0.0
    c[offsets[1:] - 1] = 0.0
    return tuple(v.astype(dtype) for v in (a, b, c, d)) + (offsets,)
