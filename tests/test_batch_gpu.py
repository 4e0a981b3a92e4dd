"""Batched solves of independent lattices of uneven size (one multi-lattice stencil pass per
application), checked lattice by lattice with the CPU oracle: FP64 true residual <= 1e-10, for the
one-launch-per-step path (the default) and the persistent kernel (GBC_PERSISTENT=1)."""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("persistent", ["1", "0"], ids=["persistent", "graphs"])
def test_batch_of_uneven_lattices(persistent, monkeypatch):
    monkeypatch.setenv("GBC_PERSISTENT", persistent)
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    o = Oracle()
    kappa, csw = 0.124, 1.5
    mass = 1 / (2 * kappa) - 4
    lattices = [(4, 4, 4, 8), (6, 6, 6, 12), (8, 8, 8, 16), (4, 6, 8, 10)]
    ctxs, ops, chis = [], [], []
    for k, dims in enumerate(lattices):
        u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 500 + k), (1, 1, 1, -1))
        c = G.Context(dims, mass, csw, t_boundary=-1, max_rhs=1)
        c.load_gauge(u)
        ctxs.append(c)
        ops.append(OracleOp(dims, u, mass, csw))
        chis.append(S.z2_noise(dims, 600 + k, cb=1).reshape(-1, 12))
    batch = G.Batch(ctxs)
    try:
        psis, res = batch.solve(chis, rsd_target=1e-10)
        for k in range(len(lattices)):
            r = chis[k] - ops[k].apply(O.OP_MEO, psis[k])
            rel = np.sqrt(ops[k].norm2(r) / ops[k].norm2(chis[k]))
            assert rel <= 1.05e-10, (lattices[k], rel, res[k])
            assert res[k]["status"] == 0
            # the same answer as the single-lattice FP64 CG
            single, _, _ = ctxs[k].solve(chis[k].reshape(1, -1, 12), solver=G.SOLVER_CG, rsd_target=1e-12)
            assert np.linalg.norm(psis[k] - single[0]) / np.linalg.norm(single[0]) < 1e-8
    finally:
        batch.close()
        for c in ctxs:
            c.close()


@pytest.mark.parametrize("sloppy", [G.PREC_HALF, G.PREC_SINGLE], ids=["f16", "f32"])
def test_tight_target_below_inner_precision(sloppy):
    """A target of 1e-12 asks the inner CGNE for reductions below what its FP32 accumulators can
    hold on this lattice; the inner solve must stop at that floor (not drift) and the FP64 outer
    loop must still reach the target, for the single-lattice and the batched solver."""
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    o = Oracle()
    kappa, csw = 0.124, 1.5
    mass = 1 / (2 * kappa) - 4
    dims = (4, 6, 8, 10)
    u = o.apply_bc(dims, o.gauge_hot(dims, 0.3, 503), (1, 1, 1, -1))
    op = OracleOp(dims, u, mass, csw)
    chi = S.z2_noise(dims, 603, cb=1).reshape(-1, 12)
    ctx = G.Context(dims, mass, csw, t_boundary=-1, max_rhs=1, sloppy_precision=sloppy)
    ctx.load_gauge(u)
    try:
        psi, res, rc = ctx.solve(chi.reshape(1, -1, 12), solver=G.SOLVER_MIXED, rsd_target=1e-12)
        r = chi - op.apply(O.OP_MEO, psi[0])
        assert np.sqrt(op.norm2(r) / op.norm2(chi)) <= 1.05e-12, res
        assert rc == 0 and res[0]["status"] == 0
        batch = G.Batch([ctx])
        try:
            psis, bres = batch.solve([chi], rsd_target=1e-12, sloppy_precision=sloppy)
        finally:
            batch.close()
        r = chi - op.apply(O.OP_MEO, psis[0])
        assert np.sqrt(op.norm2(r) / op.norm2(chi)) <= 1.05e-12, bres
        assert bres[0]["status"] == 0
    finally:
        ctx.close()


def test_persistent_kernel_matches_per_launch_path(monkeypatch):
    """The persistent kernel runs the same recursion as the per-launch path: the same solutions (to
    the FP64 target), iteration counts within a few per lattice (the reliable-update tests fall on
    every fourth iteration of a launch, not of the solve), and far fewer launches."""
    kappa, csw = 0.124, 1.5
    mass = 1 / (2 * kappa) - 4
    lattices = [(8, 8, 8, 16), (4, 4, 4, 8), (12, 12, 12, 24)]
    ctxs, chis = [], []
    for k, dims in enumerate(lattices):
        c = G.Context(dims, mass, csw, t_boundary=-1, max_rhs=1)
        c.load_gauge(G.gauge_synthetic(dims, 0.3, 900 + k, t_boundary=-1))
        ctxs.append(c)
        chis.append(S.z2_noise(dims, 950 + k, cb=1).reshape(-1, 12))
    batch = G.Batch(ctxs)
    try:
        for mode in ("0", "1"):  # warm-up: the autotuner's trial launches count as launches
            monkeypatch.setenv("GBC_PERSISTENT", mode)
            batch.solve(chis, rsd_target=1e-10)
        out = {}
        for mode in ("1", "0"):
            monkeypatch.setenv("GBC_PERSISTENT", mode)
            psis, res = batch.solve(chis, rsd_target=1e-10)
            assert all(r["status"] == 0 and r["rel_resid"] <= 1e-10 for r in res), res
            out[mode] = (psis, res)
        for k in range(len(lattices)):
            a, b = out["1"][0][k], out["0"][0][k]
            assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-8
            ia, ib = out["1"][1][k]["n_count"], out["0"][1][k]["n_count"]
            print(f"{lattices[k]}: iterations {ia} / {ib}, reliable updates {out['1'][1][k]['n_reliable']} / "
                  f"{out['0'][1][k]['n_reliable']}, outer steps {out['1'][1][k]['n_outer']} / "
                  f"{out['0'][1][k]['n_outer']} (persistent / per-launch)")
            assert abs(ia - ib) <= max(8, 0.1 * ib), (lattices[k], ia, ib)
        la, lb = out["1"][1][0]["launches"], out["0"][1][0]["launches"]
        print(f"launches per batch solve: persistent {la}, per-launch {lb}")
        assert la * 2 < lb, (la, lb)
    finally:
        batch.close()
        for c in ctxs:
            c.close()
