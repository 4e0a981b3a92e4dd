"""Multi-shift CG (gbc_solve_multishift) on the GPU: every shifted system
(M~^dag M~ + sigma) psi = chi reaches its FP64 true relative residual when recomputed with the CPU
oracle's operator, agrees with the single-shift FP64 CG solve for shift 0, and the shifted
iteration counts follow the reference recursion (one Krylov space, so every shift reports the
iterations of the last one to converge)."""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu

KAPPA, CSW = 0.115, 1.0


@pytest.fixture(scope="module")
def setup():
    from oracle import Oracle, OracleOp
    dims = (4, 4, 4, 8)
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 31), (1, 1, 1, -1))
    mass = 1 / (2 * KAPPA) - 4
    op = OracleOp(dims, u, mass, CSW)
    ctx = G.Context(dims, mass, CSW, t_boundary=-1, max_rhs=4)
    ctx.load_gauge(u)
    yield dims, op, ctx
    ctx.close()


def _rel(op, psi, chi, sigma):
    from oracle import oracle as O
    r = chi - op.apply(O.OP_MDAGM, psi) - sigma * psi
    return np.sqrt(op.norm2(r) / op.norm2(chi))


def test_shifted_residuals_meet_targets(setup):
    dims, op, ctx = setup
    chi = S.z2_noise(dims, 11, cb=1).reshape(-1, 12)
    shifts = [0.0, 0.01, 0.1, 1.0, 4.0]
    psi, res, rc = ctx.solve_multishift(chi, shifts, rsd_target=1e-10)
    assert rc == 0
    par = S.parity(dims)
    for k, sigma in enumerate(shifts):
        assert _rel(op, psi[k], chi, sigma) <= 1.5e-10, (sigma, res[k])
        assert res[k]["status"] == 0
        assert np.all(psi[k][par == 0] == 0)  # even sites of the (zeroed) outputs untouched
    # larger shifts are better conditioned: their converged solutions are smaller
    norms = [np.linalg.norm(p) for p in psi]
    assert all(norms[i] > norms[i + 1] for i in range(len(norms) - 1))


def test_shift_zero_matches_plain_cg(setup):
    dims, op, ctx = setup
    chi = S.gaussian(dims, 12, cb=1).reshape(-1, 12)
    psi, res, rc = ctx.solve_multishift(chi, [0.0, 0.5], rsd_target=1e-12)
    one, _, _ = ctx.solve(chi.reshape(1, -1, 12), solver=G.SOLVER_CG, system=G.SYS_MDAGM, rsd_target=1e-12)
    assert np.linalg.norm(psi[0] - one[0]) / np.linalg.norm(one[0]) < 1e-9


def test_per_shift_targets_and_bad_arguments(setup):
    dims, op, ctx = setup
    chi = S.z2_noise(dims, 13, cb=1).reshape(-1, 12)
    psi, res, rc = ctx.solve_multishift(chi, [0.05, 2.0], rsd_targets=[1e-6, 1e-11])
    assert rc == 0
    assert _rel(op, psi[0], chi, 0.05) <= 1.5e-6
    assert _rel(op, psi[1], chi, 2.0) <= 1.5e-11
    with pytest.raises(G.GBCError):
        ctx.solve_multishift(chi, [-1.0])


@pytest.mark.parametrize("sloppy", [G.PREC_SINGLE, G.PREC_HALF], ids=["f32", "f16"])
def test_mixed_precision_multishift(setup, sloppy):
    """The mixed-precision form (FP32 recursion, then the FP64 defect correction of every shift with
    corrections from the shifted CG in the sloppy operator): every shift meets its FP64 target as
    recomputed by the oracle, and the solutions agree with the FP64 multi-shift ones."""
    dims, op, ctx = setup
    chi = S.z2_noise(dims, 14, cb=1).reshape(-1, 12)
    shifts = [0.0, 0.02, 0.3, 2.0]
    psi, res, rc = ctx.solve_multishift(chi, shifts, rsd_target=1e-10, sloppy_precision=sloppy)
    assert rc == 0, res
    ref, _, _ = ctx.solve_multishift(chi, shifts, rsd_target=1e-12)
    for k, sigma in enumerate(shifts):
        assert _rel(op, psi[k], chi, sigma) <= 1.5e-10, (sigma, res[k])
        assert res[k]["status"] == 0 and res[k]["n_outer"] == 1
        assert np.linalg.norm(psi[k] - ref[k]) / np.linalg.norm(ref[k]) < 1e-8
