"""Pins the CPU oracle of the learned preconditioner (no reference counterpart exists):
gauge covariance of the network, linearity, and the analytic weight gradient against finite
differences of the loss."""
import numpy as np

from oracle import Oracle
from oracle.cnn import CnnOracle


def _setup(seed=0, hidden=4):
    o = Oracle()
    dims = (4, 4, 4, 4)
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 5 + seed))
    net = CnnOracle(dims, u)
    rng = np.random.default_rng(seed)
    Ws = []
    for l in range(3):
        ci = 4 if l == 0 else hidden
        co = 4 if l == 2 else hidden
        Ws.append(0.3 * (rng.standard_normal((9, co, ci)) + 1j * rng.standard_normal((9, co, ci))))
    return o, dims, u, net, Ws, rng


def test_network_is_gauge_covariant_and_linear():
    o, dims, u, net, Ws, rng = _setup()
    V = int(np.prod(dims))
    v = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    w = rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3))
    y = net.apply(v, Ws)
    assert np.allclose(net.apply(2 * v + 3j * w, Ws), 2 * y + 3j * net.apply(w, Ws))
    g = o.gauge_hot(dims, 1.0, 99)[:, 0]
    from tests.test_oracle import _gauge_transform
    ug = _gauge_transform(u, g, dims)
    netg = CnnOracle(dims, ug)
    yg = netg.apply(np.einsum("sij,saj->sai", g, v), Ws)
    assert np.abs(yg - np.einsum("sij,saj->sai", g, y)).max() < 1e-12


def test_gradient_matches_finite_differences():
    o, dims, u, net, Ws, rng = _setup(1)
    V = int(np.prod(dims))
    vs = [rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3)) for _ in range(2)]
    es = [rng.standard_normal((V, 4, 3)) + 1j * rng.standard_normal((V, 4, 3)) for _ in range(2)]
    L, G = net.loss_grad(vs, es, Ws)
    h = 1e-6
    for li, d, oo, ii in [(0, 0, 1, 2), (0, 3, 0, 0), (1, 8, 2, 3), (2, 5, 3, 1), (1, 1, 0, 0)]:
        for comp, unit in (("re", 1.0), ("im", 1j)):
            Wp = [W.copy() for W in Ws]
            Wm = [W.copy() for W in Ws]
            Wp[li][d, oo, ii] += h * unit
            Wm[li][d, oo, ii] -= h * unit
            fd = (net.loss_grad(vs, es, Wp)[0] - net.loss_grad(vs, es, Wm)[0]) / (2 * h)
            an = G[li][d, oo, ii].real if comp == "re" else G[li][d, oo, ii].imag
            assert abs(fd - an) < 1e-5 * max(1.0, abs(an)), (li, d, oo, ii, comp, fd, an)
