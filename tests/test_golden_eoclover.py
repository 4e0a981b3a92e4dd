"""Golden vectors of the even-odd clover operator and its solve (tests/golden/eoclover_4x4x4x4.npz,
made by tests/golden/make_oracle_fixture.py): the oracle rebuilt on this host, and the GPU library
through the C ABI, reproduce the recorded M~ src, M~^dag src, solution and clover log dets; the
oracle also the symmetric and the twisted-mass operator.

Tolerances: the seeded links to 1e-14 (plaquette); FP64 operators 1e-12 relative; log dets 1e-12
relative; the oracle's solution to 1e-12 residual within 1e-9 of the golden one, the GPU's (plain
FP64 CG, and the defect correction around the single-precision BiCGStab) to 1e-11 residual within
1e-8 (M~ is well conditioned here: CGNE reaches 1e-13 in 44 iterations)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_oracle_fixture as F  # noqa: E402

GOLD = np.load(os.path.join(HERE, "golden", "eoclover_4x4x4x4.npz"))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _links():
    from oracle import Oracle
    orc = Oracle()
    u = F.links(orc)
    p, t = orc.plaquette(F.DIMS, u)
    assert abs(p - GOLD["plaquette"][0]) < 1e-14 and abs(t - GOLD["plaquette"][1]) < 1e-14
    return u


def test_fixture_header():
    assert tuple(GOLD["dims"]) == F.DIMS and float(GOLD["kappa"]) == F.KAPPA and float(GOLD["csw"]) == F.CSW
    assert np.array_equal(GOLD["src"], F.source())
    assert float(GOLD["rel_resid"]) <= 1e-13


def test_oracle_reproduces_golden():
    from oracle import OracleOp
    from oracle import oracle as O
    op = OracleOp(F.DIMS, _links(), 1 / (2 * F.KAPPA) - 4, F.CSW)
    odd = F.odd_sites(F.DIMS)
    src = F.full(GOLD["src"])
    assert rel(op.apply(O.OP_MEO, src, +1, 1)[odd], GOLD["meo"]) < 1e-12
    assert rel(op.apply(O.OP_MEO, src, -1, 1)[odd], GOLD["meo_dag"]) < 1e-12
    assert rel(op.apply(O.OP_SYM, src, +1, 1)[odd], GOLD["msym"]) < 1e-12
    tw = OracleOp(F.DIMS, _links(), 1 / (2 * F.KAPPA) - 4, F.CSW, twisted_m=F.TWISTED_M)
    assert rel(tw.apply(O.OP_MEO, src, +1, 1)[odd], GOLD["meo_tw"]) < 1e-12
    psi, res = op.solve(src, solver=O.SOLVER_CG, rsd=1e-12, maxit=10000)
    assert rel(psi[odd], GOLD["psi"]) < 1e-9
    assert abs(op.logdet_even() - GOLD["logdet_even"]) < 1e-12 * abs(GOLD["logdet_even"])
    assert abs(op.logdet_odd() - GOLD["logdet_odd"]) < 1e-12 * abs(GOLD["logdet_odd"])


@pytest.mark.gpu
def test_gpu_reproduces_golden():
    from chroma_gb300 import gbclover as G
    ctx = G.Context(F.DIMS, 1 / (2 * F.KAPPA) - 4, F.CSW, t_boundary=-1, max_rhs=2)
    try:
        ctx.load_gauge(_links())
        odd = F.odd_sites(F.DIMS)
        src = F.full(GOLD["src"])
        assert rel(ctx.apply(G.OP_MEO, src, +1, 1, G.PREC_DOUBLE)[0][odd], GOLD["meo"]) < 1e-12
        assert rel(ctx.apply(G.OP_MEO, src, -1, 1, G.PREC_DOUBLE)[0][odd], GOLD["meo_dag"]) < 1e-12
        le, lo = ctx.logdet()
        assert abs(le - GOLD["logdet_even"]) < 1e-12 * abs(GOLD["logdet_even"])
        assert abs(lo - GOLD["logdet_odd"]) < 1e-12 * abs(GOLD["logdet_odd"])
        for solver in (G.SOLVER_CG, G.SOLVER_BICGSTAB):
            psi, res, rc = ctx.solve(src, solver=solver, rsd_target=1e-11, sloppy_precision=G.PREC_SINGLE)
            assert rc == 0 and res[0]["status"] == 0 and res[0]["rel_resid"] <= 1.05e-11, (solver, res)
            assert rel(psi[0][odd], GOLD["psi"]) < 1e-8, (solver, res)
    finally:
        ctx.close()
