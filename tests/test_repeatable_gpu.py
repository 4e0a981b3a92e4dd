"""Run-to-run repeatability of a mixed-precision solve: two processes that share the stencil shape
decisions (the tune cache: the first process times the shapes and records its choices, the second
reads them) give bitwise-identical solutions.  Every reduction of the solve sums in a fixed order
for a given shape, so the only source of run-to-run differences is the autotuner's timing, which
can pick another shape (whose FP32 sums round in another order) from one process to the next."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu

SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, {root!r})
from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S
dims = (8, 8, 8, 16)
ctx = G.Context(dims, 1 / (2 * 0.124) - 4, 1.5, t_boundary=-1, max_rhs=4)
ctx.load_gauge(G.gauge_synthetic(dims, 0.3, 31, t_boundary=-1))
chi = np.stack([S.z2_noise(dims, 70 + k, cb=1).reshape(-1, 12) for k in range(4)])
psi, res, rc = ctx.solve(chi, solver=G.SOLVER_BICGSTAB, rsd_target=1e-10, delta=0.01, inner_tol=1e-5)
assert rc == 0, res
np.save({out!r}, psi)
print(ctx.tune_report())
"""


def test_two_processes_give_identical_solutions(tmp_path):
    env = dict(os.environ, GBC_TUNE_CACHE=str(tmp_path / "tune.cache"))
    outs = []
    for k in range(2):
        out = str(tmp_path / f"psi{k}.npy")
        r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT, out=out)], env=env, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        outs.append(np.load(out))
    assert np.array_equal(outs[0], outs[1])


SMOKE = r"""
import sys
import numpy as np
sys.path.insert(0, {root!r})
from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S
dims = (8, 8, 8, 8)
ctx = G.Context(dims, 1 / (2 * 0.115) - 4, 1.0, t_boundary=-1, max_rhs=4)
ctx.load_gauge(G.gauge_synthetic(dims, 0.3, 2024, t_boundary=-1))
chi = S.z2_noise(dims, 5, cb=1).reshape(1, -1, 12)
psi, res, rc = ctx.solve(chi, solver=G.SOLVER_MIXED, sloppy_precision=G.PREC_HALF, rsd_target=1e-10)
chis = np.stack([S.z2_noise(dims, 6 + k, cb=1).reshape(-1, 12) for k in range(4)])
psis, bres, brc = ctx.solve(chis, solver=G.SOLVER_BICGSTAB, sloppy_precision=G.PREC_HALF, rsd_target=1e-10,
                            delta=0.01, inner_tol=1e-5)
assert rc == 0 and brc == 0
np.save({out!r}, np.concatenate([psi, psis]))
print(ctx.tune_report())
"""


def test_shipped_table_makes_the_smoke_solves_repeatable(tmp_path):
    """The smoke test's solves (8^4, kappa 0.115, c_sw 1.0) take every stencil shape from the
    shipped table, without a tune cache, so two processes give bitwise-identical solutions."""
    table = os.path.join(ROOT, "chroma_gb300", "tune", "default.tunecache")
    if not os.path.exists(table):
        pytest.skip("no shipped tune table")
    env = {k: v for k, v in os.environ.items() if k not in ("GBC_TUNE_CACHE", "GBC_TUNE_DEFAULTS", "GBC_SHAPE")}
    outs = []
    for k in range(2):
        out = str(tmp_path / f"smoke{k}.npy")
        r = subprocess.run([sys.executable, "-c", SMOKE.format(root=ROOT, out=out)], env=env, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        decisions = [line for line in r.stdout.splitlines() if "->" in line]
        assert decisions and all("(shipped table)" in line for line in decisions), r.stdout
        outs.append(np.load(out))
    assert np.array_equal(outs[0], outs[1])
