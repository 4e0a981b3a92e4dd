"""Persistent autotuning (GBC_TUNE_CACHE, the counterpart of QUDA's tunecache): a first context
times the stencil shapes and appends its decisions to the file; a second context, and a second
process, take them from the file without timing and get bitwise the same operator."""
import os
import subprocess
import sys

import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIMS = (8, 8, 8, 8)
KAPPA, CSW = 0.115, 1.0


def _apply(n=12):
    u = G.gauge_synthetic(DIMS, 0.3, 314, t_boundary=-1)
    ctx = G.Context(DIMS, 1 / (2 * KAPPA) - 4, CSW, t_boundary=-1, max_rhs=12)
    try:
        ctx.load_gauge(u)
        V = int(np.prod(DIMS))
        xs = np.stack([S.gaussian(DIMS, 500 + k).reshape(V, 12) for k in range(n)])
        y = ctx.apply(G.OP_MEO, xs, +1, 1, G.PREC_HALF)
        return y, ctx.tune_report()
    finally:
        ctx.close()


def _choices(report):
    return sorted(line.split(" (")[0] for line in report.strip().splitlines())


def test_tune_cache_roundtrip(tmp_path, monkeypatch):
    path = tmp_path / "tunecache.txt"
    monkeypatch.setenv("GBC_TUNE_CACHE", str(path))
    monkeypatch.delenv("GBC_SHAPE", raising=False)
    y1, rep1 = _apply()
    assert rep1 and "(cache)" not in rep1
    lines = path.read_text().splitlines()
    assert len(lines) == len(rep1.strip().splitlines()) >= 2
    assert all(len(line.split()) == 5 and "nrhs=12" in line for line in lines)
    # a second context of this process takes every choice from the cache
    y2, rep2 = _apply()
    assert all(line.endswith("(cache)") for line in rep2.strip().splitlines())
    assert _choices(rep1) == _choices(rep2)
    assert np.array_equal(y1, y2)
    # and so does another process
    code = ("import sys; sys.path[:0] = [%r, %r]; from test_tune_cache_gpu import _apply; "
            "_, rep = _apply(); print(rep)") % (ROOT, os.path.join(ROOT, "tests"))
    out = subprocess.run([sys.executable, "-c", code], env=dict(os.environ), capture_output=True, text=True,
                         cwd=ROOT, check=True).stdout
    assert out.strip() and all(line.endswith("(cache)") for line in out.strip().splitlines())
    assert len(path.read_text().splitlines()) == len(lines)
