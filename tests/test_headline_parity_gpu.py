"""Parity at the benchmark sizes: the 12-source propagator solves of the 32^3 x 64 workload
(kappa 0.125, c_sw 1.6) and of the 24^3 x 48 workload (kappa 0.124, c_sw 1.5), hot-start links
eps 0.3, antiperiodic t, the 12 spin-colour point sources at the origin solved as one batch of the
full system (Chroma's quarkProp4_a -> PrecFermActQprop, eoprec_fermact_qprop.cc:41-80), checked
by the oracle:

  - every source's FP64 true relative residual |chi - M psi| / |chi|, with the oracle's
    unpreconditioned operator, is <= 1e-10 (the target; 1.05e-10 allows the last-bit difference
    between the library's FP64 residual and the oracle's);
  - source 0 is also solved by the oracle itself (Chroma's InvCG2 on the Schur system, FP64, target
    1e-12) and the relative error of the GPU solution against it is reported and bounded.

These are the sizes where the stencil runs its multi-right-hand-side shapes and the solver its
reliable updates and outer FP64 steps at production scale; the operator-level parity tests run on
small lattices."""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import sources as S

pytestmark = pytest.mark.gpu

CASES = [((24, 24, 24, 48), 0.124, 1.5), ((32, 32, 32, 64), 0.125, 1.6)]
SEED = 20251203


@pytest.mark.parametrize("dims,kappa,csw", CASES, ids=["24^3x48", "32^3x64"])
def test_propagator_against_oracle(dims, kappa, csw):
    from oracle import OracleOp
    mass = 1 / (2 * kappa) - 4
    u = G.gauge_synthetic(dims, 0.3, SEED, t_boundary=-1)
    src = S.point_sources(dims).reshape(12, -1, 12)
    ctx = G.Context(dims, mass, csw, t_boundary=-1, max_rhs=12)
    try:
        ctx.load_gauge(u)
        psi, res, rc = ctx.solve(src, solver=G.SOLVER_BICGSTAB, system=G.SYS_FULL, rsd_target=1e-10,
                                 sloppy_precision=G.PREC_HALF, delta=0.01, inner_tol=1e-5)
        assert rc == 0, res
    finally:
        ctx.close()
    op = OracleOp(dims, u, mass, csw)
    rr = op.full_residuals(psi, src)
    print(f"{dims}: oracle true relative residuals max {rr.max():.3e} min {rr.min():.3e}")
    assert rr.max() <= 1.05e-10, rr
    # the library's own FP64 residual agrees with the oracle's
    lib = np.array([r["rel_resid"] for r in res])
    assert np.all(np.abs(lib - rr) <= 1e-2 * rr + 1e-16), (lib, rr)
    ref, info = op.qprop(src[0], rsd=1e-12)
    err = float(np.linalg.norm(psi[0] - ref) / np.linalg.norm(ref))
    print(f"{dims}: error of source 0 against the oracle's FP64 solve {err:.3e} "
          f"(oracle {info['n_count']} CG iterations, residual {info['rel_resid']:.2e})")
    assert info["rel_resid"] < 1e-11
    assert err < 1e-8, err
