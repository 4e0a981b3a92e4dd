"""BLAS-1 parity: the reductions and fused vector updates of the solvers, one kernel at a time,
through the C ABI (gbc_blas), against the oracle's FP64 norm2 / innerProduct over rb[1] (QDP++'s
Double sums) and the FP64 update formulas of InvCG2 and BiCGStab.

Inputs are drawn exactly representable in the storage precision of their role (FP32 values for
FP32 fields; for fp16 fields, fp16 components times a power-of-two site norm whose largest
component is the norm itself), so that GPU and oracle see identical numbers and the comparison
measures the kernels' arithmetic alone.  Tolerances (relative, over the whole output):
  reductions and FP64 / FP32 outputs   1e-12 (FP64 arithmetic), 1e-6 (FP32 arithmetic)
  fp16-stored outputs                  2e-3  (one fp16 rounding of the site-normalised value)
A field whose sites span 8 orders of magnitude bounds the FP32 thread- and warp-level sums of the
reductions (the block sums and the final sum are FP64)."""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu

PAIRS = [(G.PREC_DOUBLE, G.PREC_DOUBLE, 1e-12), (G.PREC_SINGLE, G.PREC_SINGLE, 1e-6),
         (G.PREC_SINGLE, G.PREC_HALF, 1e-6)]
PAIR_IDS = ["f64", "f32", "f32-f16"]


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def representable(x, prec):
    """x rounded to a value the storage precision holds exactly (odd sites; even sites zero)."""
    if prec == G.PREC_DOUBLE:
        return x
    if prec == G.PREC_SINGLE:
        return x.astype(np.complex64).astype(np.complex128)
    # fp16 with a per-site norm: components y * 2^k, |y| <= 1 fp16, y[0].re = 1 so the norm is 2^k
    m = np.max(np.maximum(np.abs(x.real), np.abs(x.imag)), axis=-1, keepdims=True)
    k = np.ceil(np.log2(np.where(m > 0, m, 1.0)))
    scale = 2.0 ** k
    y = x / scale
    y = y.real.astype(np.float16).astype(np.float64) + 1j * y.imag.astype(np.float16).astype(np.float64)
    live = m[..., 0] > 0
    y[..., 0] = np.where(live, 1.0 + 1j * y[..., 0].imag, y[..., 0])
    return y * scale


def fields(dims, nrhs, seed, wide=False):
    """nrhs odd-site Gaussian fields (V, 12); wide: site magnitudes spread over 1e-4 .. 1e4."""
    rng = np.random.default_rng(seed)
    V = int(np.prod(dims))
    par = S.parity(dims)
    x = rng.normal(size=(nrhs, V, 12)) + 1j * rng.normal(size=(nrhs, V, 12))
    if wide:
        x *= 10.0 ** rng.uniform(-4, 4, size=(nrhs, V, 1))
    x[:, par == 0] = 0
    return np.ascontiguousarray(x)


@pytest.fixture(scope="module", params=[((8, 8, 8, 8), 3), ((32, 32, 32, 64), 1)], ids=["8^4", "32^3x64"])
def setup(request):
    from oracle import Oracle, OracleOp
    dims, nrhs = request.param
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 77), (1, 1, 1, -1))
    op = OracleOp(dims, u, 1 / (2 * 0.125) - 4, 1.6)  # its norm2 / innerProduct over rb[1]
    ctx = G.Context(dims, 1 / (2 * 0.125) - 4, 1.6, t_boundary=-1, max_rhs=max(nrhs, 3))
    yield dims, nrhs, op, ctx
    ctx.close()


@pytest.mark.parametrize("wide", [False, True], ids=["gauss", "wide"])
@pytest.mark.parametrize("pa,po,tol", PAIRS, ids=PAIR_IDS)
def test_norm2_and_cdot(setup, pa, po, tol, wide):
    dims, nrhs, op, ctx = setup
    x = representable(fields(dims, nrhs, 1, wide), po)
    got = ctx.blas(G.BLAS_NORM2, [x], prec_acc=pa, prec_op=po)
    want = np.array([op.norm2(x[r]) for r in range(nrhs)])
    assert rel(got[:, 0], want) < tol
    xa = representable(fields(dims, nrhs, 2, wide), pa)
    y = representable(fields(dims, nrhs, 3, wide), po)
    got = ctx.blas(G.BLAS_CDOT, [xa, y], prec_acc=pa, prec_op=po)
    want = np.array([op.inner(xa[r], y[r]) for r in range(nrhs)])
    # bound the error by the sum of |x||y| (the cancellation-free scale of the sum)
    scale = np.array([np.sum(np.abs(xa[r]) * np.abs(y[r])) for r in range(nrhs)])
    err = np.abs(got[:, 0] + 1j * got[:, 1] - want)
    assert np.all(err <= tol * scale), (err, scale)


@pytest.mark.parametrize("pa,po,tol", PAIRS, ids=PAIR_IDS)
def test_cg_update(setup, pa, po, tol):
    dims, nrhs, op, ctx = setup
    x = representable(fields(dims, nrhs, 4), pa)
    p = representable(fields(dims, nrhs, 5), po)
    r = representable(fields(dims, nrhs, 6, wide=True), pa)
    q = representable(fields(dims, nrhs, 7), po)
    a = np.array([0.37, -1.25, 2.5][:nrhs])
    x_want = x + a[:, None, None] * p
    r_want = r - a[:, None, None] * q
    xg, rg = x.copy(), r.copy()
    got = ctx.blas(G.BLAS_CG_UPDATE, [xg, p, rg, q], coef=a, prec_acc=pa, prec_op=po)
    assert rel(xg, x_want) < tol
    assert rel(rg, r_want) < tol
    want = np.array([op.norm2(r_want[k]) for k in range(nrhs)])
    assert rel(got[:, 0], want) < tol


@pytest.mark.parametrize("pa,po,tol", PAIRS, ids=PAIR_IDS)
def test_xpay(setup, pa, po, tol):
    dims, nrhs, op, ctx = setup
    r = representable(fields(dims, nrhs, 8), pa)
    p = representable(fields(dims, nrhs, 9), po)
    b = np.array([0.5, 1.75, -0.3][:nrhs])
    want = r + b[:, None, None] * p
    pg = p.copy()
    ctx.blas(G.BLAS_XPAY, [r, pg], coef=b, prec_acc=pa, prec_op=po)
    assert rel(pg, want) < (2e-3 if po == G.PREC_HALF else tol)


@pytest.mark.parametrize("pa,po,tol", PAIRS, ids=PAIR_IDS)
def test_bicgstab_update(setup, pa, po, tol):
    dims, nrhs, op, ctx = setup
    x = representable(fields(dims, nrhs, 10), pa)
    r = representable(fields(dims, nrhs, 11, wide=True), pa)
    p = representable(fields(dims, nrhs, 12), po)
    v = representable(fields(dims, nrhs, 13), po)
    t = representable(fields(dims, nrhs, 14), po)
    r0 = representable(fields(dims, nrhs, 15), pa)
    alpha = np.array([0.3 - 0.2j, -0.7 + 0.1j, 1.1 + 0.4j][:nrhs])
    omega = np.array([0.9 + 0.05j, 0.2 - 0.6j, -0.4 - 0.3j][:nrhs])
    coef = np.stack([alpha.real, alpha.imag, omega.real, omega.imag], axis=1).ravel()
    A, W = alpha[:, None, None], omega[:, None, None]
    s = r - A * v
    x_want = x + A * p + W * s
    r_want = s - W * t
    xg, rg = x.copy(), r.copy()
    got = ctx.blas(G.BLAS_BICG_XR, [xg, rg, p, v, t, r0], coef=coef, prec_acc=pa, prec_op=po)
    assert rel(xg, x_want) < tol
    assert rel(rg, r_want) < tol
    rr = np.array([op.norm2(r_want[k]) for k in range(nrhs)])
    assert rel(got[:, 0], rr) < tol
    dot = np.array([op.inner(r0[k], r_want[k]) for k in range(nrhs)])
    scale = np.array([np.sum(np.abs(r0[k]) * np.abs(r_want[k])) for k in range(nrhs)])
    assert np.all(np.abs(got[:, 1] + 1j * got[:, 2] - dot) <= tol * scale)


def test_blas_refuses_bad_arguments(setup):
    dims, nrhs, op, ctx = setup
    x = fields(dims, nrhs, 1)
    with pytest.raises(G.GBCError):
        ctx.blas(G.BLAS_BICG_XR, [x] * 6, coef=np.zeros(4 * nrhs), prec_acc=G.PREC_HALF, prec_op=G.PREC_HALF)
