"""The symmetric even-odd operator M_s = 1 - 1/4 A_oo^-1 D_oe A_ee^-1 D_eo (SEOPREC_CLOVER,
seoprec_clover_linop_w.cc:145-187) on the GPU against the CPU oracle: operator parity in FP64 / FP32
/ FP16 (1e-12 / 1e-6 / 5e-3 relative), the odd clover inverse, solves of M_s psi = chi and of
M_s^dag M_s psi = chi that reach the oracle's FP64 residual 1e-10, and the same with a twisted-mass
term."""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu

KAPPA, CSW = 0.12, 1.3
TOL = {G.PREC_DOUBLE: 1e-12, G.PREC_SINGLE: 1e-6, G.PREC_HALF: 5e-3}


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def setup():
    from oracle import Oracle, OracleOp
    dims = (4, 6, 4, 8)
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 808), (1, 1, 1, -1))
    mass = 1 / (2 * KAPPA) - 4
    op = OracleOp(dims, u, mass, CSW)
    ctx = G.Context(dims, mass, CSW, t_boundary=-1, max_rhs=4)
    ctx.load_gauge(u)
    yield dims, op, ctx
    ctx.close()


@pytest.mark.parametrize("prec", [G.PREC_DOUBLE, G.PREC_SINGLE, G.PREC_HALF], ids=["f64", "f32", "f16"])
def test_symmetric_operator_matches_oracle(setup, prec):
    from oracle import oracle as O
    dims, op, ctx = setup
    V = int(np.prod(dims))
    par = S.parity(dims)
    xs = np.stack([S.gaussian(dims, 60 + k).reshape(V, 12) for k in range(3)])
    for gop, oop, isign in [(G.OP_SYM, O.OP_SYM, 1), (G.OP_SYM, O.OP_SYM, -1), (G.OP_SYM_MDAGM, O.OP_SYM_MDAGM, 1),
                            (G.OP_CLOVINV, O.OP_CLOVER_INV, 1)]:
        got = ctx.apply(gop, xs, isign, 1, prec)
        for k in range(3):
            want = op.apply(oop, xs[k], isign, 1)
            err = rel(got[k][par == 1], want[par == 1])
            assert err < TOL[prec], (gop, isign, prec, k, err)


@pytest.mark.parametrize("solver,sloppy,system", [(G.SOLVER_CG, 0, G.SYS_SYM), (G.SOLVER_MIXED, G.PREC_HALF, G.SYS_SYM),
                                                  (G.SOLVER_FGMRES, G.PREC_SINGLE, G.SYS_SYM),
                                                  (G.SOLVER_MIXED, G.PREC_HALF, G.SYS_SYM_MDAGM),
                                                  (G.SOLVER_BICGSTAB, G.PREC_HALF, G.SYS_SYM)],
                         ids=["cg64", "mixed16", "fgmres32", "mdagm-mixed16", "bicgstab16"])
def test_symmetric_solves(setup, solver, sloppy, system):
    from oracle import oracle as O
    dims, op, ctx = setup
    chi = S.z2_noise(dims, 70, cb=1).reshape(1, -1, 12)
    psi, res, rc = ctx.solve(chi, solver=solver, system=system, rsd_target=1e-10, sloppy_precision=sloppy)
    oop = O.OP_SYM if system == G.SYS_SYM else O.OP_SYM_MDAGM
    r = chi[0] - op.apply(oop, psi[0], +1, 1)
    assert np.sqrt(op.norm2(r) / op.norm2(chi[0])) <= 1.05e-10, res
    assert rc == 0 and res[0]["status"] == 0
    # the symmetric and asymmetric systems have the same solution up to A_oo: M_s psi = chi
    # <=> M~ psi = A_oo chi
    if system == G.SYS_SYM:
        a_chi = op.apply(O.OP_CLOVER, chi[0], +1, 1)
        psi2, _, _ = ctx.solve(a_chi.reshape(1, -1, 12), solver=G.SOLVER_CG, system=G.SYS_MEO, rsd_target=1e-12)
        assert rel(psi[0], psi2[0]) < 1e-8


def test_factory_selects_symmetric_operator(setup):
    """The solver factory with a SEOPREC_CLOVER action solves M_s psi = chi."""
    from oracle import oracle as O
    from chroma_gb300 import syssolver as SS
    dims, op, ctx = setup
    xml = f"""<InvertParam><invType>GB300_CLOVER_INVERTER</invType><SolverType>MIXED</SolverType>
      <CloverParams><Kappa>{KAPPA}</Kappa><clovCoeff>{CSW}</clovCoeff></CloverParams>
      <RsdTarget>1e-10</RsdTarget><MaxIter>5000</MaxIter><AntiPeriodicT>true</AntiPeriodicT></InvertParam>"""
    from oracle import Oracle
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 808), (1, 1, 1, -1))
    solver = SS.TheLinOpFermSystemSolverFactory.createObject("GB300_CLOVER_INVERTER", xml, ".", u, dims,
                                                              operator="SEOPREC_CLOVER")
    chi = S.gaussian(dims, 71, cb=1).reshape(-1, 12)
    psi, res = solver(np.zeros_like(chi), chi)
    r = chi - op.apply(O.OP_SYM, psi, +1, 1)
    assert np.sqrt(op.norm2(r) / op.norm2(chi)) <= 1.05e-10
    solver.ctx.close()


@pytest.mark.parametrize("prec", [G.PREC_DOUBLE, G.PREC_SINGLE, G.PREC_HALF], ids=["f64", "f32", "f16"])
def test_symmetric_twisted_operator_and_solves(prec):
    """M_s + isign i mu gamma_5 (seoprec_clover_linop_w.cc:174-184; the clover term and its inverses
    carry no twist) against the oracle for both isigns, and solves of M psi = chi and
    M^dag M psi = chi that reach the oracle's FP64 residual 1e-10."""
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    dims = (4, 6, 4, 8)
    mu = 0.05
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 809), (1, 1, 1, -1))
    mass = 1 / (2 * KAPPA) - 4
    op = OracleOp(dims, u, mass, CSW, twisted_m=mu)
    ctx = G.Context(dims, mass, CSW, t_boundary=-1, max_rhs=3, twisted_m=mu)
    try:
        ctx.load_gauge(u)
        V = int(np.prod(dims))
        par = S.parity(dims)
        xs = np.stack([S.gaussian(dims, 90 + k).reshape(V, 12) for k in range(3)])
        for gop, oop, isign in [(G.OP_SYM, O.OP_SYM, 1), (G.OP_SYM, O.OP_SYM, -1),
                                (G.OP_SYM_MDAGM, O.OP_SYM_MDAGM, 1)]:
            got = ctx.apply(gop, xs, isign, 1, prec)
            for k in range(3):
                want = op.apply(oop, xs[k], isign, 1)
                assert rel(got[k][par == 1], want[par == 1]) < TOL[prec], (gop, isign, k)
        if prec != G.PREC_DOUBLE:
            return
        chi = S.z2_noise(dims, 91, cb=1).reshape(1, -1, 12)
        for solver, sloppy, system, oop in [(G.SOLVER_BICGSTAB, G.PREC_HALF, G.SYS_SYM, O.OP_SYM),
                                            (G.SOLVER_MIXED, G.PREC_HALF, G.SYS_SYM_MDAGM, O.OP_SYM_MDAGM)]:
            psi, res, rc = ctx.solve(chi, solver=solver, system=system, rsd_target=1e-10, sloppy_precision=sloppy)
            assert rc == 0, res
            r = chi[0] - op.apply(oop, psi[0], +1, 1)
            assert np.sqrt(op.norm2(r) / op.norm2(chi[0])) <= 1.05e-10
    finally:
        ctx.close()
