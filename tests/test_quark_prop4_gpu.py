"""The batched propagator hook (syssolver.quark_prop4, the counterpart of quarkProp4_a that
chroma_plugin's quarkProp4GB300 provides) on the device: every column of the solution propagator
solves M psi = chi for its spin-colour source to the FP64 true residual 1e-10 of the oracle's
unpreconditioned operator, with one batched device solve for the 12 sources."""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import syssolver as SS

pytestmark = pytest.mark.gpu

XML = """
<InvertParam>
  <invType>GB300_CLOVER_INVERTER</invType>
  <CloverParams><Kappa>0.124</Kappa><clovCoeff>1.5</clovCoeff></CloverParams>
  <RsdTarget>1e-10</RsdTarget>
  <MaxIter>5000</MaxIter>
  <SolverType>BICGSTAB</SolverType>
  <Delta>0.01</Delta>
  <InnerTol>1e-5</InnerTol>
  <CudaSloppyPrecision>HALF</CudaSloppyPrecision>
  <AntiPeriodicT>true</AntiPeriodicT>
</InvertParam>
"""


def test_quark_prop4_columns_solve_their_sources():
    from oracle import OracleOp
    dims = (8, 8, 8, 16)
    V = int(np.prod(dims))
    u = G.gauge_synthetic(dims, 0.3, 606, t_boundary=-1)
    params = SS.SysSolverGB300CloverParams.from_xml(XML)
    solver = SS.PrecFermActQprop(u, dims, params)
    rng = np.random.default_rng(9)
    q_src = rng.normal(size=(V, 4, 4, 3, 3)) + 1j * rng.normal(size=(V, 4, 4, 3, 3))
    q_src *= 10.0 ** rng.uniform(-3, 3)  # quarkProp4_a normalises each source: any scale works
    q_sol, ncg, results = SS.quark_prop4(solver, q_src)
    assert len(results) == 12 and all(r.status == 0 for r in results)
    op = OracleOp(dims, u, params.CloverParams.Mass, params.CloverParams.clovCoeffR)
    for c in range(3):
        for s in range(4):
            chi = q_src[:, :, s, :, c].reshape(V, 12)
            psi = q_sol[:, :, s, :, c].reshape(V, 12)
            rr = op.full_residuals(psi, chi)[0]
            assert rr <= 1.05e-10, (c, s, rr)
