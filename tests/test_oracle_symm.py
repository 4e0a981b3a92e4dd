"""The oracle's symmetric and asymmetric even-odd clover operators against the identities of Chroma's
mainprogs/tests/symm_prec_tests.cc, on its actions (symm_prec_xml.h:16-90: Mass 0.1, clovCoeff 1,
two stout steps with rho 0.14 orthogonal to t, boundary (1, 1, 1, -1), TwistedM 0.05 for the
twisted operator) and a hot gauge field:

- CheckOp (:107-160): A_oo M_s = M~ for PLUS, M_s^dag A_oo^dag = M~^dag for MINUS;
- TestLogDetUnitGauge (:633-653): log det A_ee = log det A_oo on the unit gauge;
- TestLogDetShiftedGauge (:655-693): log det A_oo of U equals log det A_ee of U shifted by one
  site in t (and the other way round), per site to 1e-13;
- TestTwist (:695-761): M(mu) = M_s + i mu gamma_5, M(mu)^dag = M_s^dag - i mu gamma_5 and
  M(mu)^dag M(mu) = M_s^dag M_s + mu^2 + i mu (M_s^dag gamma_5 - gamma_5 M_s).
"""
import numpy as np
import pytest

from oracle import Oracle, OracleOp
from oracle import oracle as O

DIMS = (4, 4, 4, 8)
MASS, CSW, MU = 0.1, 1.0, 0.05
G5 = np.repeat(np.array([1, 1, -1, -1]), 3)  # gamma_5 of the DeGrand-Rossi basis, per spin-colour


def _parity(dims):
    s = np.arange(int(np.prod(dims)))
    x = s % dims[0]
    y = (s // dims[0]) % dims[1]
    z = (s // (dims[0] * dims[1])) % dims[2]
    t = s // (dims[0] * dims[1] * dims[2])
    return (x + y + z + t) % 2


ODD = _parity(DIMS) == 1


@pytest.fixture(scope="module")
def orc():
    return Oracle()


@pytest.fixture(scope="module")
def thin(orc):
    return orc.gauge_hot(DIMS, 1.0, 123)


def _state(orc, u):
    """STOUT_FERM_STATE: two stout steps (rho 0.14, not in t), then the fermion boundary."""
    return orc.apply_bc(DIMS, orc.stout(DIMS, u, 0.14, 2, smear_dirs=(1, 1, 1, 0)), (1, 1, 1, -1))


@pytest.fixture(scope="module")
def links(orc, thin):
    return _state(orc, thin)


def _gaussian_odd(seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((ODD.size, 12)) + 1j * rng.standard_normal((ODD.size, 12))
    v[~ODD] = 0
    return v


def test_check_op(links):
    op = OracleOp(DIMS, links, MASS, CSW)
    x = _gaussian_odd(1)
    nx = np.linalg.norm(x)
    # PLUS: A_oo (M_s x) = M~ x
    am = op.apply(O.OP_CLOVER, op.apply(O.OP_SYM, x, +1, 1), +1, 1)
    d = op.apply(O.OP_MEO, x, +1, 1) - am
    assert np.linalg.norm(d[~ODD]) == 0
    assert np.linalg.norm(d[ODD]) < 1e-14 * nx
    # MINUS: M_s^dag (A_oo^dag x) = M~^dag x
    ma = op.apply(O.OP_SYM, op.apply(O.OP_CLOVER, x, -1, 1), -1, 1)
    d = op.apply(O.OP_MEO, x, -1, 1) - ma
    assert np.linalg.norm(d[~ODD]) == 0
    assert np.linalg.norm(d[ODD]) < 1e-14 * nx


def test_logdet_unit_gauge(orc):
    V = int(np.prod(DIMS))
    unit = np.broadcast_to(np.eye(3, dtype=np.complex128), (V, 4, 3, 3)).copy()
    op = OracleOp(DIMS, _state(orc, unit), MASS, CSW)
    assert abs(op.logdet_even() - op.logdet_odd()) < 1e-14
    assert abs(op.logdet_even() - V // 2 * 12 * np.log(4 + MASS)) < 1e-12 * op.logdet_even()


def test_logdet_shifted_gauge(orc, thin, links):
    # shift(u, FORWARD, 3): u'(x) = u(x + t^); the site index runs t slowest
    L = DIMS
    shifted = np.roll(thin.reshape(L[3], L[2] * L[1] * L[0], 4, 3, 3), -1, axis=0).reshape(thin.shape)
    op = OracleOp(DIMS, links, MASS, CSW)
    op_s = OracleOp(DIMS, _state(orc, shifted), MASS, CSW)
    vh = int(np.prod(DIMS)) // 2
    # the log det of the symmetric operator's A_ee is the asymmetric operator's (one clover term)
    assert abs(op.logdet_even() - op.logdet_odd()) / vh > 1e-6  # a hot field: the parities differ
    assert abs(op.logdet_even() - op_s.logdet_odd()) / vh < 1e-13
    assert abs(op.logdet_odd() - op_s.logdet_even()) / vh < 1e-13


def test_twist(links):
    op = OracleOp(DIMS, links, MASS, CSW)
    tw = OracleOp(DIMS, links, MASS, CSW, twisted_m=MU)
    x = _gaussian_odd(2)
    nx = np.linalg.norm(x)
    g5x = 1j * G5 * x
    # PLUS: M(mu) x = M_s x + i mu gamma_5 x
    d = op.apply(O.OP_SYM, x, +1, 1) + MU * g5x - tw.apply(O.OP_SYM, x, +1, 1)
    assert np.linalg.norm(d[ODD]) < 1e-14 * nx
    # MINUS: M(mu)^dag x = M_s^dag x - i mu gamma_5 x
    d = op.apply(O.OP_SYM, x, -1, 1) - MU * g5x - tw.apply(O.OP_SYM, x, -1, 1)
    assert np.linalg.norm(d[ODD]) < 1e-14 * nx
    # M(mu)^dag M(mu) = M_s^dag M_s + mu^2 + i mu M_s^dag gamma_5 - i mu gamma_5 M_s
    want = op.apply(O.OP_SYM, op.apply(O.OP_SYM, x, +1, 1), -1, 1) + MU * MU * x
    want += MU * op.apply(O.OP_SYM, g5x, -1, 1)
    want -= MU * 1j * G5 * op.apply(O.OP_SYM, x, +1, 1)
    for got in (tw.apply(O.OP_SYM, tw.apply(O.OP_SYM, x, +1, 1), -1, 1), tw.apply(O.OP_SYM_MDAGM, x, +1, 1)):
        assert np.linalg.norm((got - want)[ODD]) < 1e-13 * nx
