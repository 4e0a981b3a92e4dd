"""Double-float arithmetic on the FP64 fields (GBC_PREC_DF64: each value hi + lo in two floats),
the arithmetic of the intermediate defect-correction residuals of full-system solves (and of the
Schur prep of the solvers that iterate on it directly).

  - every operator block in this arithmetic against the oracle (FP64): relative error <= 1e-12
    over the output field (the same bound as the FP64 kernels; double-float carries ~48 bits),
    and against the FP64 kernels;
  - a field whose site magnitudes span 1e-12 .. 1e4 (the range of a propagator's tails): the
    same bound, so the exponent handling of the conversions holds;
  - full-system solves with the double-float outer steps (the default) and with FP64 outer steps
    (GBC_OUTER_DF=0): both reach the FP64 true residual checked by the oracle, with the same
    solution to the target's precision and iteration counts within a few."""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu

KAPPA, CSW = 0.124, 1.5


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def setup():
    from oracle import Oracle, OracleOp
    dims = (8, 8, 8, 8)
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 4321), (1, 1, 1, -1))
    mass = 1 / (2 * KAPPA) - 4
    op = OracleOp(dims, u, mass, CSW)
    ctx = G.Context(dims, mass, CSW, t_boundary=-1, max_rhs=12)
    ctx.load_gauge(u)
    yield dims, op, ctx
    ctx.close()


@pytest.mark.parametrize("wide", [False, True], ids=["gauss", "wide"])
@pytest.mark.parametrize("isign", [1, -1])
def test_operators_in_double_float(setup, isign, wide):
    from oracle import oracle as O
    dims, op, ctx = setup
    V = int(np.prod(dims))
    x = S.gaussian(dims, 11).reshape(V, 12)
    if wide:
        x = x * (10.0 ** np.random.default_rng(5).uniform(-12, 4, size=(V, 1)))
    cases = [(G.OP_DSLASH, O.OP_DSLASH, 0), (G.OP_DSLASH, O.OP_DSLASH, 1), (G.OP_CLOVER, O.OP_CLOVER, 1),
             (G.OP_CLOVINV, O.OP_CLOVER_INV, 0), (G.OP_MEO, O.OP_MEO, 1), (G.OP_UNPREC, O.OP_UNPREC, 0)]
    if isign == 1:
        cases.append((G.OP_MDAGM, O.OP_MDAGM, 1))
    par = S.parity(dims)
    for gop, oop, cb in cases:
        want = op.apply(oop, x, isign, cb)
        got = ctx.apply(gop, x, isign, cb, G.PREC_DF64)[0]
        f64 = ctx.apply(gop, x, isign, cb, G.PREC_DOUBLE)[0]
        sel = slice(None) if gop == G.OP_UNPREC else (par == cb)
        err, err64 = rel(got[sel], want[sel]), rel(f64[sel], want[sel])
        print(f"op {gop} cb {cb} isign {isign}: double-float {err:.2e}, FP64 {err64:.2e}")
        assert err < 1e-12, (gop, cb, isign, err)


def test_symmetric_operator_refuses_double_float(setup):
    dims, op, ctx = setup
    x = S.gaussian(dims, 3).reshape(-1, 12)
    with pytest.raises(G.GBCError):
        ctx.apply(G.OP_SYM, x, 1, 1, G.PREC_DF64)


def test_full_solve_with_double_float_outer_steps(monkeypatch):
    from oracle import Oracle, OracleOp
    dims = (8, 8, 8, 16)
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 99), (1, 1, 1, -1))
    mass = 1 / (2 * KAPPA) - 4
    op = OracleOp(dims, u, mass, CSW)
    src = S.point_sources(dims).reshape(12, -1, 12)
    ctx = G.Context(dims, mass, CSW, t_boundary=-1, max_rhs=12)
    try:
        ctx.load_gauge(u)
        out = {}
        for mode in ("1", "0"):
            monkeypatch.setenv("GBC_OUTER_DF", mode)
            psi, res, rc = ctx.solve(src, solver=G.SOLVER_BICGSTAB, system=G.SYS_FULL, rsd_target=1e-10,
                                     sloppy_precision=G.PREC_HALF, delta=0.01, inner_tol=1e-5)
            assert rc == 0, res
            rr = op.full_residuals(psi, src)
            print(f"GBC_OUTER_DF={mode}: oracle residual max {rr.max():.2e}, "
                  f"iterations {[r['n_count'] for r in res]}")
            assert rr.max() <= 1.05e-10
            out[mode] = (psi, res)
        (a, ra), (b, rb) = out["1"], out["0"]
        assert rel(a, b) < 1e-8
        for x, y in zip(ra, rb):
            assert abs(x["n_count"] - y["n_count"]) <= max(10, 0.15 * y["n_count"])
    finally:
        ctx.close()
