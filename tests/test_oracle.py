"""Pins the CPU oracle against the reference's known answers and analytic identities.

- NERSC archive KAT: Chroma's tests/t_asqtad_prop/t_nersc.cfg header (PLAQUETTE, LINK_TRACE),
  reproduced from the committed payload (tests/golden/nersc_4x4x4x4.npz) with the 12-real
  reconstruction row3 = conj(row1 x row2).
- Free field: with U = 1 the unpreconditioned operator is diagonal on plane waves,
  M = (4+m) - sum cos p + i sum gamma sin p (lwldslash_w.h:16-44, eoprec_linop.h:147-165).
- gamma_5 hermiticity of the even-odd operator (PLUS vs MINUS of eoprec_clover_linop_w.cc:142-187).
- Gauge covariance of the hopping term, the clover term and the even-odd operator.
- Clover term equal to diag_mass - sum_{mu<nu} (c/2) gamma_mu gamma_nu F_{mu nu}
  (clover_term_qdp_w.h:299-396 comment, makeClov :398-553) built from explicit gamma matrices.
- Unit-gauge log det = Vh * 12 * log(4+m) (symm_prec_tests.cc:633-652).
- LDL^dag inverse: A A^-1 = 1 on the even sites.
- The full system's outer residual taken from the original source equals chi'_o - M~ x and the
  odd part of chi - M psi (eoprec_fermact_qprop.cc:47-76).
- Solvers: CG / reliable CG / FGMRES converge; the Schur-complement propagator solves the full system.
"""
import io
import os
import tempfile

import numpy as np
import pytest

from oracle import Oracle, OracleOp
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def orc():
    return Oracle()


def coords(dims):
    V = int(np.prod(dims))
    s = np.arange(V)
    x = s % dims[0]
    y = (s // dims[0]) % dims[1]
    z = (s // (dims[0] * dims[1])) % dims[2]
    t = s // (dims[0] * dims[1] * dims[2])
    return np.stack([x, y, z, t], axis=1)


def parity(dims):
    return coords(dims).sum(axis=1) % 2


def rand_spinor(dims, seed, cb=None):
    rng = np.random.default_rng(seed)
    V = int(np.prod(dims))
    v = rng.standard_normal((V, 12)) + 1j * rng.standard_normal((V, 12))
    if cb is not None:
        v[parity(dims) != cb] = 0
    return v


def test_nersc_known_answer(orc):
    fx = np.load(os.path.join(HERE, "golden", "nersc_4x4x4x4.npz"))
    dims = [int(d) for d in fx["dims"]]
    hdr = "BEGIN_HEADER\n"
    for i, d in enumerate(dims):
        hdr += f"DIMENSION_{i + 1} = {d}\n"
    hdr += f"PLAQUETTE = {float(fx['plaquette'])!r}\nLINK_TRACE = {float(fx['link_trace'])!r}\n"
    hdr += f"DATATYPE = {str(fx['datatype'])}\nFLOATING_POINT = {str(fx['floating_point'])}\nEND_HEADER\n"
    with tempfile.NamedTemporaryFile(suffix=".cfg", delete=False) as f:
        f.write(hdr.encode() + fx["payload"].tobytes())
        path = f.name
    try:
        d, u, p_hdr, t_hdr = orc.read_nersc(path)
    finally:
        os.unlink(path)
    assert list(d) == dims
    plaq, tr = orc.plaquette(dims, u)
    # the header carries 10 significant digits of a sum formed from IEEE32 data
    assert abs(plaq - 0.0382422893) < 2e-9
    assert abs(tr - 0.4630322094) < 2e-9
    uu = np.einsum("sxij,sxkj->sxik", u, u.conj())
    assert np.abs(uu - np.eye(3)).max() < 1e-6


def test_gamma_basis(orc):
    g, g5 = orc.gamma()
    for m in range(4):
        assert np.allclose(g[m], g[m].conj().T)
        for n in range(4):
            assert np.allclose(g[m] @ g[n] + g[n] @ g[m], 2 * np.eye(4) * (m == n))
    assert np.allclose(g5, np.diag([1, 1, -1, -1]))


def test_hot_start_unitary_and_seeded(orc):
    dims = (4, 4, 4, 4)
    u = orc.gauge_hot(dims, 0.3, 7)
    u2 = orc.gauge_hot(dims, 0.3, 7)
    u3 = orc.gauge_hot(dims, 0.3, 8)
    assert np.array_equal(u, u2) and not np.array_equal(u, u3)
    uu = np.einsum("sxij,sxkj->sxik", u, u.conj())
    assert np.abs(uu - np.eye(3)).max() < 1e-14
    assert np.abs(np.linalg.det(u) - 1).max() < 1e-14


def test_stout_keeps_su3_and_smooths(orc):
    dims = (4, 4, 4, 8)
    u = orc.gauge_hot(dims, 0.3, 3)
    us = orc.stout(dims, u, 0.1, 4)
    uu = np.einsum("sxij,sxkj->sxik", us, us.conj())
    assert np.abs(uu - np.eye(3)).max() < 1e-13
    assert np.abs(np.linalg.det(us) - 1).max() < 1e-13
    assert orc.plaquette(dims, us)[0] > orc.plaquette(dims, u)[0] + 0.05
    # spatial-only smearing leaves the time links untouched
    u3 = orc.stout(dims, u, 0.1, 2, smear_dirs=(1, 1, 1, 0))
    assert np.array_equal(u3[:, 3], u[:, 3]) and not np.allclose(u3[:, 0], u[:, 0])


def test_free_field_plane_wave(orc):
    dims = (4, 4, 4, 8)
    V = int(np.prod(dims))
    u = np.broadcast_to(np.eye(3, dtype=np.complex128), (V, 4, 3, 3)).copy()
    u = orc.apply_bc(dims, u, (1, 1, 1, -1))
    kappa = 0.115
    m = 1 / (2 * kappa) - 4
    op = OracleOp(dims, u, m, 1.0)
    g, _ = orc.gamma()
    X = coords(dims)
    rng = np.random.default_rng(0)
    for n in [(0, 0, 0, 0), (1, 0, 2, 3), (3, 1, 1, 7)]:
        p = np.array([2 * np.pi * n[0] / dims[0], 2 * np.pi * n[1] / dims[1], 2 * np.pi * n[2] / dims[2],
                      (2 * n[3] + 1) * np.pi / dims[3]])
        eta = rng.standard_normal((4, 3)) + 1j * rng.standard_normal((4, 3))
        phase = np.exp(1j * (X @ p))
        psi = phase[:, None, None] * eta[None]
        Mk = (4 + m - np.cos(p).sum()) * np.eye(4) + 1j * sum(g[k] * np.sin(p[k]) for k in range(4))
        want = phase[:, None, None] * (Mk @ eta)[None]
        got = op.apply(O.OP_UNPREC, psi.reshape(V, 12)).reshape(V, 4, 3)
        assert np.abs(got - want).max() < 1e-13


def test_gamma5_hermiticity(orc):
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 11))
    op = OracleOp(dims, u, 1 / (2 * 0.115) - 4, 1.0)
    x = rand_spinor(dims, 1, cb=1)
    y = rand_spinor(dims, 2, cb=1)
    lhs = op.inner(x, op.apply(O.OP_MEO, y, +1))
    rhs = np.conj(op.inner(y, op.apply(O.OP_MEO, x, -1)))
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
    # unpreconditioned: gamma5 M gamma5 = M^dag (MINUS)
    g5 = np.repeat(np.array([1, 1, -1, -1]), 3)
    z = rand_spinor(dims, 3)
    a = g5 * op.apply(O.OP_UNPREC, g5 * z, +1)
    b = op.apply(O.OP_UNPREC, z, -1)
    assert np.abs(a - b).max() < 1e-12


def _gauge_transform(u, g, dims):
    V = int(np.prod(dims))
    X = coords(dims)
    ug = np.empty_like(u)
    for mu in range(4):
        Y = X.copy()
        Y[:, mu] = (Y[:, mu] + 1) % dims[mu]
        sp = Y[:, 0] + dims[0] * (Y[:, 1] + dims[1] * (Y[:, 2] + dims[2] * Y[:, 3]))
        ug[:, mu] = g @ u[:, mu] @ np.conj(np.transpose(g[sp], (0, 2, 1)))
    return ug


def test_gauge_covariance(orc):
    dims = (4, 4, 4, 8)
    V = int(np.prod(dims))
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 21))
    g = orc.gauge_hot(dims, 1.0, 22)[:, 0]
    ug = _gauge_transform(u, g, dims)
    m = 1 / (2 * 0.12) - 4
    op = OracleOp(dims, u, m, 1.2)
    opg = OracleOp(dims, ug, m, 1.2)
    psi = rand_spinor(dims, 5).reshape(V, 4, 3)
    psig = np.einsum("sij,saj->sai", g, psi)
    for code, cb in [(O.OP_DSLASH, 0), (O.OP_DSLASH, 1), (O.OP_CLOVER, 1), (O.OP_CLOVER_INV, 0), (O.OP_MEO, 1)]:
        a = opg.apply(code, psig.reshape(V, 12), +1, cb).reshape(V, 4, 3)
        b = np.einsum("sij,saj->sai", g, op.apply(code, psi.reshape(V, 12), +1, cb).reshape(V, 4, 3))
        assert np.abs(a - b).max() < 1e-12, code


def _unpack_block(row):
    """Full 12x12 matrix (index spin*3+colour) from one packed site (72 reals)."""
    diag = row[:12].reshape(2, 6)
    offd = row[12:].view(np.complex128).reshape(2, 15)
    A = np.zeros((12, 12), dtype=np.complex128)
    for b in range(2):
        B = np.diag(diag[b]).astype(np.complex128)
        k = 0
        for i in range(6):
            for j in range(i):
                B[i, j] = offd[b, k]
                B[j, i] = np.conj(offd[b, k])
                k += 1
        A[6 * b:6 * b + 6, 6 * b:6 * b + 6] = B
    return A


def test_clover_matches_sigma_F(orc):
    dims = (4, 4, 4, 4)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.4, 31))
    csw = 1.3
    m = 0.05
    op = OracleOp(dims, u, m, csw)
    clov, inv = op.clover()
    F = orc.mesfield(dims, u)
    g, _ = orc.gamma()
    pairs = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    for s in [0, 5, 77, 200, 255]:
        A = (4 + m) * np.eye(12, dtype=np.complex128)
        for k, (mu, nu) in enumerate(pairs):
            A -= 0.5 * csw * np.kron(g[mu] @ g[nu], F[s, k])
        assert np.abs(_unpack_block(clov[s]) - A).max() < 1e-13
    # A^-1 on even sites
    par = parity(dims)
    for s in np.nonzero(par == 0)[0][:8]:
        assert np.abs(_unpack_block(clov[s]) @ _unpack_block(inv[s]) - np.eye(12)).max() < 1e-13


def test_unit_gauge_logdet(orc):
    dims = (4, 4, 4, 8)
    V = int(np.prod(dims))
    u = orc.apply_bc(dims, np.broadcast_to(np.eye(3, dtype=np.complex128), (V, 4, 3, 3)).copy())
    m = 0.1
    op = OracleOp(dims, u, m, 1.0)
    want = V // 2 * 12 * np.log(4 + m)
    assert abs(op.logdet_even() - want) < 1e-13 * want


def test_schur_complement_identity(orc):
    """M~ psi_o equals the odd part of M (psi_o + psi_e) with psi_e = -A_ee^-1 M_eo psi_o, times nothing else."""
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 41))
    op = OracleOp(dims, u, 1 / (2 * 0.12) - 4, 1.0)
    psi_o = rand_spinor(dims, 6, cb=1)
    # psi_e = A_ee^-1 (1/2 D_eo psi_o)  =>  (M psi)_e = 0
    psi_e = op.apply(O.OP_CLOVER_INV, 0.5 * op.apply(O.OP_DSLASH, psi_o, +1, 0), +1, 0)
    full = op.apply(O.OP_UNPREC, psi_o + psi_e)
    par = parity(dims)
    assert np.abs(full[par == 0]).max() < 1e-12
    meo = op.apply(O.OP_MEO, psi_o)
    assert np.abs(full[par == 1] - meo[par == 1]).max() < 1e-12


def test_outer_residual_from_the_original_source(orc):
    """The defect correction's residual of the full system, taken from the original source
    (r = chi_o - A_oo x + 1/2 D_oe A_ee^-1 (chi_e + 1/2 D_eo x)), equals chi'_o - M~ x for the
    Schur-prepared chi'_o = chi_o + 1/2 D_oe A_ee^-1 chi_e (eoprec_fermact_qprop.cc:47-54), and the
    odd part of chi - M psi for psi reconstructed from x (:60-76), whose even part vanishes."""
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 43))
    op = OracleOp(dims, u, 1 / (2 * 0.124) - 4, 1.5)
    par = parity(dims)
    chi = rand_spinor(dims, 7)
    chi_e, chi_o = chi * (par == 0)[:, None], chi * (par == 1)[:, None]
    x = rand_spinor(dims, 8, cb=1)
    chip = chi_o + 0.5 * op.apply(O.OP_DSLASH, op.apply(O.OP_CLOVER_INV, chi_e, +1, 0), +1, 1)
    want = chip - op.apply(O.OP_MEO, x)
    ue = op.apply(O.OP_CLOVER_INV, chi_e + 0.5 * op.apply(O.OP_DSLASH, x, +1, 0), +1, 0)
    got = chi_o - op.apply(O.OP_CLOVER, x, +1, 1) + 0.5 * op.apply(O.OP_DSLASH, ue, +1, 1)
    odd = par == 1
    scale = np.abs(want[odd]).max()
    assert np.abs(got[odd] - want[odd]).max() < 1e-13 * scale
    full = chi - op.apply(O.OP_UNPREC, x + ue)
    assert np.abs(full[odd] - got[odd]).max() < 1e-13 * scale
    assert np.abs(full[par == 0]).max() < 1e-13 * scale


def test_symmetric_operator_identities(orc):
    """The symmetric operator M_s = 1 - 1/4 A_oo^-1 D_oe A_ee^-1 D_eo (seoprec_clover_linop_w.cc:
    145-187) is A_oo^-1 M~; its MINUS application is its adjoint; A_oo A_oo^-1 = 1 on the odd
    sites; OP_SYM_MDAGM = M_s^dag M_s."""
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 43))
    op = OracleOp(dims, u, 1 / (2 * 0.12) - 4, 1.3)
    x = rand_spinor(dims, 8, cb=1)
    y = rand_spinor(dims, 9, cb=1)
    par = parity(dims)
    ms = op.apply(O.OP_SYM, x, +1, 1)
    want = op.apply(O.OP_CLOVER_INV, op.apply(O.OP_MEO, x), +1, 1)
    assert np.abs(ms[par == 1] - want[par == 1]).max() < 1e-12 * np.abs(want).max()
    back = op.apply(O.OP_CLOVER, op.apply(O.OP_CLOVER_INV, x, +1, 1), +1, 1)
    assert np.abs(back[par == 1] - x[par == 1]).max() < 1e-12
    msd = op.apply(O.OP_SYM, y, -1, 1)
    lhs = op.inner(y, ms)
    rhs = op.inner(msd, x)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)
    mm = op.apply(O.OP_SYM_MDAGM, x, +1, 1)
    want = op.apply(O.OP_SYM, ms, -1, 1)
    assert np.abs(mm[par == 1] - want[par == 1]).max() < 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("solver", [O.SOLVER_CG, O.SOLVER_RELIABLE_CG, O.SOLVER_FGMRES, O.SOLVER_BICGSTAB])
def test_solvers_converge(orc, solver):
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 51))
    op = OracleOp(dims, u, 1 / (2 * 0.115) - 4, 1.0)
    chi = rand_spinor(dims, 7, cb=1)
    psi, res = op.solve(chi, solver=solver, rsd=1e-10, maxit=2000, delta=0.1, nkrylov=16)
    assert res["n_count"] > 0
    r = chi - op.apply(O.OP_MEO, psi)
    true_rel = np.sqrt(op.norm2(r) / op.norm2(chi))
    assert abs(true_rel - res["rel_resid"]) < 1e-3 * true_rel + 1e-16
    assert true_rel < 5e-9


def test_reliable_bicgstab_reaches_fp64_target(orc):
    # the mixed single/double reliable BiCGStab (the pattern of the GPU inner solver) reaches a
    # 1e-10 FP64 true residual and the CG solution
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 53), (1, 1, 1, -1))
    op = OracleOp(dims, u, 1 / (2 * 0.12) - 4, 1.2)
    chi = rand_spinor(dims, 10, cb=1)
    x_cg, _ = op.solve(chi, solver=O.SOLVER_CG, rsd=1e-12, maxit=5000)
    x_rb, r_rb = op.solve(chi, solver=O.SOLVER_RELIABLE_BICGSTAB, rsd=1e-10, maxit=5000, delta=0.1)
    assert r_rb["n_count"] > 0 and r_rb["rel_resid"] <= 1.05e-10, r_rb
    assert np.linalg.norm(x_rb - x_cg) < 1e-8 * np.linalg.norm(x_cg)


def test_richardson_multiprec_defect_correction(orc):
    # InvMultiPrecRichardson with a single-precision BiCGStab inner solve to 1e-5 (the outer pattern
    # of the GPU mixed solvers): FP64 true residual 1e-10 in a few outer steps, the CG solution
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 54), (1, 1, 1, -1))
    op = OracleOp(dims, u, 1 / (2 * 0.12) - 4, 1.2)
    chi = rand_spinor(dims, 11, cb=1)
    x_cg, _ = op.solve(chi, solver=O.SOLVER_CG, rsd=1e-12, maxit=5000)
    x_rm, r_rm = op.solve(chi, solver=O.SOLVER_RICHARDSON_BICGSTAB, rsd=1e-10, maxit=5000, delta=1e-5)
    assert r_rm["rel_resid"] <= 1.05e-10, r_rm
    assert 2 <= r_rm["n_outer"] <= 4, r_rm
    assert np.linalg.norm(x_rm - x_cg) < 1e-8 * np.linalg.norm(x_cg)


def test_bicgstab_matches_cg(orc):
    # BiCGStab on M~ (no normal equations) and CGNE reach the same solution, BiCGStab in fewer
    # operator applications (2 per iteration for both)
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 52))
    op = OracleOp(dims, u, 1 / (2 * 0.12) - 4, 1.2)
    chi = rand_spinor(dims, 9, cb=1)
    x_cg, r_cg = op.solve(chi, solver=O.SOLVER_CG, rsd=1e-12, maxit=5000)
    x_bi, r_bi = op.solve(chi, solver=O.SOLVER_BICGSTAB, rsd=1e-12, maxit=5000)
    assert 0 < r_bi["n_count"] < r_cg["n_count"], (r_bi, r_cg)
    assert np.linalg.norm(x_bi - x_cg) < 1e-9 * np.linalg.norm(x_cg)


def test_qprop_full_residual(orc):
    dims = (4, 4, 4, 8)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 61))
    op = OracleOp(dims, u, 1 / (2 * 0.115) - 4, 1.0)
    chi = rand_spinor(dims, 8)
    psi, res = op.qprop(chi, rsd=1e-11)
    r = op.apply(O.OP_UNPREC, psi) - chi
    assert np.sqrt((np.abs(r) ** 2).sum() / (np.abs(chi) ** 2).sum()) < 1e-9
    assert res["rel_resid"] < 1e-9


def test_twisted_mass_term(orc):
    dims = (4, 4, 4, 4)
    u = orc.apply_bc(dims, orc.gauge_hot(dims, 0.3, 71))
    m = 0.1
    op0 = OracleOp(dims, u, m, 1.0)
    op1 = OracleOp(dims, u, m, 1.0, twisted_m=0.05)
    x = rand_spinor(dims, 9, cb=1)
    g5 = np.repeat(np.array([1, 1, -1, -1]), 3)
    for isign in (+1, -1):
        d = op1.apply(O.OP_MEO, x, isign) - op0.apply(O.OP_MEO, x, isign)
        assert np.abs(d - isign * 0.05j * g5 * x).max() < 1e-13
