"""The oracle's FGMRES pieces against the fixtures of Chroma's mainprogs/tests/fgmres_dr_tests.cc:
the flexible Arnoldi cycle (arnoldi5 :162-249, arnoldi5GivensRot :377-524), the Givens rotation's
special cases (:251-375), the triangular least-squares solve (:527-567) and the full solve at the
fixture's targets (testFullSolverNoDeflate :569-604, targets 1e-3 and 1e-9 from :648-650, with
the fixture's MR preconditioner, RsdMR 0.1 and MaxMR 10).

The operator is the fixture's action (:10-46): anisotropic clover, Kappa 0.115, clovCoeffR 0.91,
clovCoeffT 1.07, xi_0 2.464, nu 0.95, two stout steps with rho 0.22 orthogonal to t, boundary
(1, 1, 1, -1), on a hot gauge field.
"""
import numpy as np
import pytest

from oracle import Oracle, OracleOp
from oracle import oracle as O

DIMS = (4, 4, 4, 8)
NK = 5


def _parity(dims):
    s = np.arange(int(np.prod(dims)))
    x = s % dims[0]
    y = (s // dims[0]) % dims[1]
    z = (s // (dims[0] * dims[1])) % dims[2]
    t = s // (dims[0] * dims[1] * dims[2])
    return (x + y + z + t) % 2


ODD = _parity(DIMS) == 1


@pytest.fixture(scope="module")
def op():
    orc = Oracle()
    u = orc.stout(DIMS, orc.gauge_hot(DIMS, 1.0, 97), 0.22, 2, smear_dirs=(1, 1, 1, 0))
    u = orc.apply_bc(DIMS, u, (1, 1, 1, -1))
    return OracleOp(DIMS, u, 1 / (2 * 0.115) - 4, 0.91, 1.07, aniso=True, xi_0=2.464, nu=0.95, t_dir=3)


def _gaussian_odd(seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((ODD.size, 12)) + 1j * rng.standard_normal((ODD.size, 12))
    v[~ODD] = 0
    return v


def _replay_rotations(H, beta, dim):
    """arnoldi5GivensRot: for each column j apply the rotations of columns 0..j-1, then make the
    rotation of column j and apply it to the column and to |chi| e_0."""
    Hr = H.copy()
    res = np.zeros(H.shape[1], dtype=np.complex128)
    res[0] = beta
    made_on = []  # column i as it was when rotation i was made
    for j in range(dim):
        for i in range(j):
            M = Hr.copy()
            M[i] = made_on[i]
            M, _ = O.givens(M, i, [j])
            Hr[j] = M[j]
        made_on.append(Hr[j].copy())
        Hr, res = O.givens(Hr, j, [j], res)
    return Hr, res


@pytest.mark.parametrize("rsd", [1e-6, 1e-3, 1e-9, 0.9])
def test_flexible_arnoldi_cycle(op, rsd):
    chi = _gaussian_odd(11)
    beta = np.sqrt(op.norm2(chi))
    Vs, H, R, g, dim = op.arnoldi(chi, NK, rsd)
    assert 1 <= dim <= NK
    if rsd <= 1e-3:
        assert dim == NK  # arnoldi5: five columns do not reach these targets
    # the cycle stops at the first column whose accumulated residual |g_{j+1}| meets the target
    assert abs(g[dim].real) <= rsd * beta or dim == NK
    assert all(abs(g[j].real) > rsd * beta for j in range(1, dim))
    # upper Hessenberg: H(col, row) = 0 exactly for row > col + 1
    for col in range(NK):
        assert np.all(H[col, col + 2:] == 0)
    # v_0 .. v_dim orthonormal on the odd sites and zero on the even ones (one modified Gram-Schmidt
    # pass: orthogonality drifts to ~1e-13 over five columns; the fixture allows |(v_i, v_j)|^2 < 1e-16)
    assert np.all(Vs[: dim + 1][:, ~ODD] == 0)
    vo = Vs[: dim + 1][:, ODD].reshape(dim + 1, -1)
    gram = vo.conj() @ vo.T
    assert np.abs(np.diag(gram) - 1).max() < 1e-14
    assert np.abs(gram - np.diag(np.diag(gram))).max() < 1e-11
    # Arnoldi relation M~ v_j = sum_{i <= j+1} H(j, i) v_i
    for j in range(dim):
        av = op.apply(O.OP_MEO, Vs[j])[ODD].reshape(-1)
        assert np.linalg.norm(av - H[j, : j + 2] @ vo[: j + 2]) < 1e-13 * np.linalg.norm(av)
    # fresh rotations triangularise H and reproduce the cycle's R bit for bit, and its g up to the
    # rounding of |chi| (the oracle's threaded sums may add in another order)
    Hr, res = _replay_rotations(H, beta, dim)
    for row in range(1, dim + 1):
        assert np.all(Hr[:row, row] == 0)
    assert np.array_equal(Hr[:dim], R[:dim])
    assert np.abs(res - g).max() <= 1e-14 * beta
    # the least-squares update x = V eta has true residual |g_dim|
    eta = O.least_squares(R, g, dim)
    r = chi - op.apply(O.OP_MEO, np.tensordot(eta, Vs[:dim], axes=1))
    assert abs(np.sqrt(op.norm2(r)) - abs(g[dim])) < 1e-12 * beta


def _rand_c(rng):
    return complex(rng.uniform(-1, 1), rng.uniform(-1, 1))


def test_givens_f0_g0():
    H, _ = O.givens(np.zeros((1, 2)), 0, [0])
    assert np.all(H == 0)


def test_givens_f0_gnot0():
    g = _rand_c(np.random.default_rng(1))
    H = np.zeros((1, 2), dtype=np.complex128)
    H[0, 1] = g
    H, _ = O.givens(H, 0, [0])
    assert H[0, 1] == 0 and H[0, 0] == g


def test_givens_fnot0_g0():
    f = _rand_c(np.random.default_rng(2))
    H = np.zeros((1, 2), dtype=np.complex128)
    H[0, 0] = f
    H, _ = O.givens(H, 0, [0])
    assert H[0, 1] == 0 and H[0, 0] == np.sqrt(abs(f) ** 2)


def test_givens_fnot0_gnot0():
    rng = np.random.default_rng(3)
    f, g = _rand_c(rng), _rand_c(rng)
    H = np.array([[f, g], [f, g]])
    H, _ = O.givens(H, 0, [0, 1])
    assert H[0, 1] == 0
    assert abs(H[1, 1]) < 1e-15 * abs(f) * abs(g) * 4
    assert abs(H[0, 0].real - H[1, 0].real) < 1e-15 * abs(H[0, 0]) * 4


def test_givens_rejects_bad_columns():
    with pytest.raises(ValueError):
        O.givens(np.zeros((2, 2)), 1, [1])  # no row below column 1
    with pytest.raises(ValueError):
        O.givens(np.zeros((2, 3)), 0, [2])


def test_least_squares():
    rng = np.random.default_rng(4)
    n_rows, n_cols = 4, 3
    R = np.zeros((n_cols, n_rows), dtype=np.complex128)
    for row in range(n_rows - 1):
        for col in range(row, n_cols):
            R[col, row] = _rand_c(rng)
    b = np.array([_rand_c(rng) for _ in range(n_rows)])
    x = O.least_squares(R, b, n_cols)
    for row in range(n_cols):
        prod = sum(R[col, row] * x[col] for col in range(row, n_cols))
        assert abs(prod - b[row]) < 1e-13 * max(1.0, abs(b[row]))


def _mr_preconditioner(op, rsd_mr=0.1, max_mr=10):
    """Minimal-residual steps on M~ from a zero guess, |r| <= rsd_mr |b| or max_mr steps."""
    def apply(b):
        x = np.zeros_like(b)
        r = b.copy()
        target = rsd_mr * np.sqrt(op.norm2(b))
        for _ in range(max_mr):
            if np.sqrt(op.norm2(r)) <= target:
                break
            ar = op.apply(O.OP_MEO, r)
            a = op.inner(ar, r) / op.norm2(ar)
            x += a * r
            r -= a * ar
        return x
    return apply


@pytest.mark.parametrize("rsd", [1e-3, 1e-9])
@pytest.mark.parametrize("precond", ["none", "mr"])
def test_full_solver_no_deflate(op, rsd, precond):
    chi = _gaussian_odd(12)
    pc = _mr_preconditioner(op) if precond == "mr" else None
    psi, res = op.solve(chi, solver=O.SOLVER_FGMRES, rsd=rsd, maxit=500, nkrylov=NK, precond=pc)
    r = op.apply(O.OP_MEO, psi) - chi
    rel = np.sqrt(op.norm2(r) / op.norm2(chi))
    assert rel <= rsd and abs(rel - res["rel_resid"]) <= 1e-6 * rel
