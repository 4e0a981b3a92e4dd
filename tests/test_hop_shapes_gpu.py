"""Every compiled launch shape of the hopping kernels, pinned one at a time with GBC_SHAPE, against
the CPU oracle: FP16 storage (5e-3 relative), 1 and 12 right-hand sides, both isigns.

The two-sites-per-thread fp16 kernel pairs cb sites i and i + Vh/2, i.e. (x, y, z, t) with
(x', y, z, t + Lt/2); lattices with odd Lt/2 (4x6x4x6, 6x4x8x10) give the paired site the other
x parity and so exercise the index arithmetic of both cases.  The two-right-hand-sides-per-thread
kernels (shapes 12-15) run only for even nrhs: their pins apply to the 12-RHS cases."""
import os

import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu

KAPPA = 0.115
CSW = 1.0
NUM_SHAPES = 16  # the candidates compiled into the library (kHopShapes)


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _context(dims, u, mass, shape):
    # the pin is read when a context first launches each kernel variant (and then cached there);
    # the callers remove it again once the context is closed
    os.environ["GBC_SHAPE"] = str(shape)
    ctx = G.Context(dims, mass, CSW, t_boundary=-1, max_rhs=12)
    ctx.load_gauge(u)
    return ctx


@pytest.mark.parametrize("dims", [(4, 4, 4, 8), (4, 6, 4, 6), (6, 4, 8, 10)], ids=["4x4x4x8", "4x6x4x6", "6x4x8x10"])
def test_every_shape_matches_oracle(dims):
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 4321), (1, 1, 1, -1))
    mass = 1 / (2 * KAPPA) - 4
    op = OracleOp(dims, u, mass, CSW)
    V = int(np.prod(dims))
    xs = np.stack([S.gaussian(dims, 900 + k).reshape(V, 12) for k in range(12)])
    par = S.parity(dims)
    cases = [(G.OP_DSLASH, O.OP_DSLASH, 0), (G.OP_DSLASH, O.OP_DSLASH, 1), (G.OP_MEO, O.OP_MEO, 1),
             (G.OP_MDAGM, O.OP_MDAGM, 1)]
    want = {}
    for gop, oop, cb in cases:
        for isign in (1, -1):
            if gop == G.OP_MDAGM and isign == -1:
                continue
            want[(gop, cb, isign)] = [op.apply(oop, xs[k], isign, cb) for k in range(12)]
    try:
        for shape in range(NUM_SHAPES):
            ctx = _context(dims, u, mass, shape)
            try:
                for (gop, cb, isign), w in want.items():
                    for n in (1, 12):
                        got = ctx.apply(gop, xs[:n], isign, cb, G.PREC_HALF)
                        for k in range(n):
                            err = rel(got[k][par == cb], w[k][par == cb])
                            assert err < 5e-3, (shape, gop, cb, isign, n, k, err)
            finally:
                ctx.close()
    finally:
        os.environ.pop("GBC_SHAPE", None)


@pytest.mark.parametrize("shape", [6, 7, 8])
def test_pair_kernel_mixed_solve(shape):
    """A mixed FP16/FP64 solve whose stencil (and its fused |M psi|^2 reduction) runs on one of the
    two-sites-per-thread shapes reaches the FP64 true residual 1e-10 of the oracle operator."""
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    dims = (4, 6, 4, 6)
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 77), (1, 1, 1, -1))
    mass = 1 / (2 * KAPPA) - 4
    op = OracleOp(dims, u, mass, CSW)
    chi = S.z2_noise(dims, 5, cb=1).reshape(1, -1, 12)
    try:
        ctx = _context(dims, u, mass, shape)
        try:
            psi, res, rc = ctx.solve(chi, solver=G.SOLVER_MIXED, rsd_target=1e-10)
        finally:
            ctx.close()
    finally:
        os.environ.pop("GBC_SHAPE", None)
    r = chi[0] - op.apply(O.OP_MEO, psi[0])
    assert np.sqrt(op.norm2(r) / op.norm2(chi[0])) <= 1.05e-10
    assert rc == 0 and res[0]["status"] == 0


@pytest.mark.parametrize("solver", [G.SOLVER_MIXED, G.SOLVER_BICGSTAB], ids=["cgne", "bicgstab"])
@pytest.mark.parametrize("shape", [12, 13, 14, 15])
def test_rhs_pair_kernel_mixed_solve(shape, solver):
    """A 12-RHS mixed FP16/FP64 solve whose stencil (and its fused |M psi|^2, or BiCGStab's (t, s),
    (t, t), reduction) runs on one of the two-right-hand-sides-per-thread shapes: every solution
    reaches the FP64 true residual 1e-10 of the oracle operator."""
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    dims = (4, 6, 4, 6)
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 78), (1, 1, 1, -1))
    mass = 1 / (2 * KAPPA) - 4
    op = OracleOp(dims, u, mass, CSW)
    chi = np.stack([S.z2_noise(dims, 40 + k, cb=1).reshape(-1, 12) for k in range(12)])
    try:
        ctx = _context(dims, u, mass, shape)
        try:
            psi, res, rc = ctx.solve(chi, solver=solver, rsd_target=1e-10, delta=0.01 if solver == G.SOLVER_BICGSTAB
                                     else 0.1)
        finally:
            ctx.close()
    finally:
        os.environ.pop("GBC_SHAPE", None)
    assert rc == 0
    for k in range(12):
        r = chi[k] - op.apply(O.OP_MEO, psi[k])
        assert np.sqrt(op.norm2(r) / op.norm2(chi[k])) <= 1.05e-10, k
        assert res[k]["status"] == 0
