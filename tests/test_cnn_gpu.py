"""GPU parity of the learned preconditioner's kernels against the CPU oracle (oracle/cnn.py).

Tolerances: the channel mixing runs BF16 x BF16 -> FP32 on the tensor cores, so outputs agree
to 2e-2 relative (norm over the field) and gradients to 5e-2 relative (norm over all weights).
"""
import os
import tempfile

import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    from oracle import Oracle
    from oracle.cnn import CnnOracle
    dims = (4, 4, 4, 8)
    o = Oracle()
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 31), (1, 1, 1, -1))
    ctx = G.Context(dims, 1 / (2 * 0.12) - 4, 1.0, t_boundary=-1, max_rhs=4)
    ctx.load_gauge(u)
    ctx.precond_init(hidden=12, layers=4, seed=3)
    yield dims, ctx, CnnOracle(dims, u)
    ctx.close()


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _perturbed_weights(ctx, seed):
    rng = np.random.default_rng(seed)
    w = ctx.precond_weights()
    w = w + 0.05 * rng.standard_normal(w.size).astype(np.float32)
    ctx.precond_set_weights(w)
    return w


def test_forward_matches_oracle(setup):
    from oracle.cnn import unpack_weights
    dims, ctx, net = setup
    w = _perturbed_weights(ctx, 1)
    Ws = unpack_weights(w)
    V = int(np.prod(dims))
    x = np.stack([S.gaussian(dims, 10 + k, cb=1).reshape(V, 12) for k in range(3)])
    got = ctx.precond_apply(x)
    for k in range(3):
        want = net.apply(x[k], Ws).reshape(V, 12)
        assert _rel(got[k], want) < 2e-2, k
    par = S.parity(dims)
    assert np.all(got[:, par == 0] == 0)


def test_loss_and_gradient_match_oracle(setup):
    from oracle.cnn import unpack_weights
    dims, ctx, net = setup
    w = _perturbed_weights(ctx, 2)
    Ws = unpack_weights(w)
    V = int(np.prod(dims))
    xs = np.stack([S.gaussian(dims, 20 + k, cb=1).reshape(V, 12) for k in range(2)])
    es = np.stack([S.gaussian(dims, 30 + k, cb=1).reshape(V, 12) for k in range(2)])
    loss, g = ctx.precond_loss_grad(xs, es)
    oloss, og = net.loss_grad(list(xs), list(es), Ws)
    assert abs(loss - oloss) < 2e-2 * oloss
    ogf = np.concatenate([x.reshape(-1) for x in og])
    gz = g[0::2] + 1j * g[1::2]
    assert _rel(gz, ogf) < 5e-2


def test_training_reduces_loss(setup):
    dims, ctx, net = setup
    V = int(np.prod(dims))
    ctx.precond_init(hidden=12, layers=4, seed=5)
    xs = np.stack([S.gaussian(dims, 40 + k, cb=1).reshape(V, 12) for k in range(8)])
    # a learnable target: a fixed covariant map of the input (the oracle network at other weights)
    from oracle.cnn import unpack_weights
    w_true = ctx.precond_weights() + 0.1 * np.random.default_rng(9).standard_normal(
        ctx.precond_weights().size).astype(np.float32)
    Wt = unpack_weights(w_true)
    es = np.stack([net.apply(x, Wt).reshape(V, 12) for x in xs])
    losses = ctx.precond_train(xs, es, epochs=30, batch=4, lr=3e-3)
    assert losses[-1] < 0.5 * losses[0], losses


def test_weights_file_roundtrip_and_corruption(setup):
    dims, ctx, net = setup
    w = ctx.precond_weights()
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "w.gbcw")
        ctx.precond_save(p)
        ctx.precond_set_weights(np.zeros_like(w))
        ctx.load_precond(p)
        assert np.array_equal(ctx.precond_weights(), w)
        raw = bytearray(open(p, "rb").read())
        raw[40] ^= 0xFF
        open(p, "wb").write(bytes(raw))
        with pytest.raises(G.GBCError) as e:
            ctx.load_precond(p)
        assert e.value.code == 8  # GBC_ERR_PRECOND
        with pytest.raises(G.GBCError):
            ctx.load_precond(os.path.join(d, "missing.gbcw"))
    assert np.array_equal(ctx.precond_weights(), w)  # a failed load keeps the previous network


def test_fgmres_with_network_converges(setup):
    from oracle import OracleOp
    from oracle import oracle as O
    dims, ctx, net = setup
    V = int(np.prod(dims))
    # an untrained network starts as (nearly) the identity map
    ctx.precond_init(hidden=12, layers=4, seed=11)
    chi = S.z2_noise(dims, 3, cb=1).reshape(1, V, 12)
    psi, res, rc = ctx.solve(chi, solver=G.SOLVER_FGMRES, use_precond=1, rsd_target=1e-10)
    assert rc == 0, res
    op = OracleOp(dims, net.u, 1 / (2 * 0.12) - 4, 1.0)
    r = chi[0] - op.apply(O.OP_MEO, psi[0])
    assert np.sqrt(op.norm2(r) / op.norm2(chi[0])) <= 1.05e-10


def test_trained_network_cuts_fgmres_iterations():
    """The committed network (trained on 16^3 x 32, kappa 0.115, c_sw 1.0) on a gauge configuration
    outside its training set: FGMRES(16) with it needs at most 3/4 of the iterations without it,
    and both solutions meet the oracle's FP64 true residual 1e-10."""
    from oracle import OracleOp
    from oracle import oracle as O
    weights = os.path.join(os.path.dirname(G.__file__), "weights", "cnn_16x16x16x32_k0.115_csw1.0.gbcw")
    dims = (16, 16, 16, 32)
    V = int(np.prod(dims))
    mass = 1 / (2 * 0.115) - 4
    u = G.gauge_synthetic(dims, 0.3, 999_999, t_boundary=-1)
    ctx = G.Context(dims, mass, 1.0, t_boundary=-1, max_rhs=1)
    try:
        ctx.load_gauge(u)
        ctx.load_precond(weights)
        chi = S.z2_noise(dims, 77, cb=1).reshape(1, V, 12)
        sols, its = [], []
        for use in (0, 1):
            psi, res, rc = ctx.solve(chi, solver=G.SOLVER_FGMRES, use_precond=use, rsd_target=1e-10,
                                     sloppy_precision=G.PREC_SINGLE)
            assert rc == 0, res
            sols.append(psi[0])
            its.append(res[0]["n_count"])
    finally:
        ctx.close()
    assert its[1] <= 0.75 * its[0], its
    op = OracleOp(dims, u, mass, 1.0)
    for psi in sols:
        r = chi[0] - op.apply(O.OP_MEO, psi)
        assert np.sqrt(op.norm2(r) / op.norm2(chi[0])) <= 1.05e-10
