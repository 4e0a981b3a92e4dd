"""Stout smearing on the GPU (gbc_stout_smear, FP64) against the CPU oracle's restatement of
stout_utils.cc: the same algorithm in FP64, so the smeared links agree to rounding (1e-12)."""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,dirs,nsteps,rho", [((4, 4, 4, 8), (1, 1, 1, 1), 4, 0.1),
                                                  ((6, 4, 8, 6), (1, 1, 1, 0), 3, 0.1),
                                                  ((4, 4, 4, 4), (1, 1, 1, 1), 2, 0.25)],
                         ids=["4x4x4x8-all", "6x4x8x6-stout3d", "4^4-rho0.25"])
def test_stout_matches_oracle(dims, dirs, nsteps, rho):
    from oracle import Oracle
    o = Oracle()
    u = o.gauge_hot(dims, 0.3, 2024)
    want = o.stout(dims, u, rho, nsteps, smear_dirs=dirs)
    got = G.stout_smear(dims, u, nsteps, rho, dirs)
    assert np.max(np.abs(got - want)) < 1e-12
    # the links of directions that are not smeared are unchanged
    for mu in range(4):
        if not dirs[mu]:
            assert np.array_equal(got[:, mu], u[:, mu])
    # unitarity is kept
    uu = np.einsum("vmij,vmkj->vmik", got, got.conj())
    assert np.max(np.abs(uu - np.eye(3))) < 1e-12


def test_stout_then_solve_matches_host_generator():
    """Links smeared on the GPU give the same operator as the host generator's smeared links:
    a solve on either reaches the oracle's FP64 residual 1e-10."""
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    from chroma_gb300 import sources as S
    o = Oracle()
    dims = (4, 4, 4, 8)
    thin = G.gauge_synthetic(dims, 0.2, 77, t_boundary=1)
    host = G.gauge_synthetic(dims, 0.2, 77, n_stout=4, rho=0.1, t_boundary=1)
    dev = G.stout_smear(dims, thin, 4, 0.1)
    assert np.max(np.abs(dev - host)) < 1e-12
    u = o.apply_bc(dims, dev, (1, 1, 1, -1))
    mass = 1 / (2 * 0.12) - 4
    op = OracleOp(dims, u, mass, 1.2)
    ctx = G.Context(dims, mass, 1.2, t_boundary=-1, max_rhs=1)
    try:
        ctx.load_gauge(u)
        chi = S.gaussian(dims, 5, cb=1).reshape(1, -1, 12)
        psi, res, rc = ctx.solve(chi, solver=G.SOLVER_MIXED, rsd_target=1e-10)
        r = chi[0] - op.apply(O.OP_MEO, psi[0])
        assert np.sqrt(op.norm2(r) / op.norm2(chi[0])) <= 1.05e-10
    finally:
        ctx.close()


def test_stout_rejects_bad_geometry():
    u = np.zeros((16, 4, 3, 3), dtype=np.complex128)
    with pytest.raises(G.GBCError):
        G.stout_smear((1, 4, 2, 2), u, 1, 0.1)
