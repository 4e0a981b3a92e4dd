"""Failure handling and dispatch of the Chroma-shaped solvers, on the CPU with a scripted stand-in for
the device context (the library's own solve is covered by the GPU tests):

- a relative residual above RsdToleranceFactor * RsdTarget (status GBC_ERR_NOT_CONVERGED) aborts
  unless SilentFail is set (syssolver_linop_clover_quda_w.h:636-643): here ``SolverFailure``;
- a BackupSolverParam group makes the LinOp solvers run the backup solver with the primary's
  clover action on the same context, and its result (iterations added) is the one returned (Chroma's QUDA clover solver reads the group,
  syssolver_quda_clover_params.cc:105-115, without running it; this adapter runs it);
- the MdagM solver's chronological predictor supplies the initial guess (syssolver_mdagm.h:32-34);
- a SEOPREC_CLOVER action selects the symmetric systems; multi-RHS sources return one result each.
"""
import numpy as np
import pytest

from chroma_gb300 import gbclover as G
from chroma_gb300 import syssolver as SS

DIMS = (4, 4, 4, 8)
V = int(np.prod(DIMS))

XML = """
<InvertParam>
  <invType>GB300_CLOVER_INVERTER</invType>
  <CloverParams>
    <Kappa>0.115</Kappa><clovCoeffR>1.1</clovCoeffR><clovCoeffT>0.9</clovCoeffT>
    <AnisoParam><anisoP>true</anisoP><t_dir>3</t_dir><xi_0>2.0</xi_0><nu>0.95</nu></AnisoParam>
  </CloverParams>
  <RsdTarget>1e-10</RsdTarget>
  <MaxIter>300</MaxIter>
  <SolverType>BICGSTAB</SolverType>
  <CudaSloppyPrecision>HALF</CudaSloppyPrecision>
  <RsdToleranceFactor>10</RsdToleranceFactor>
  {silent}
  {backup}
</InvertParam>
"""

BACKUP = """<BackupSolverParam>
    <invType>GB300_CLOVER_INVERTER</invType>
    <CloverParams><Kappa>0.2</Kappa><clovCoeff>3.0</clovCoeff></CloverParams>
    <RsdTarget>1e-11</RsdTarget><MaxIter>9000</MaxIter><SolverType>CG</SolverType>
    <CudaSloppyPrecision>DOUBLE</CudaSloppyPrecision>
  </BackupSolverParam>"""


class FakeContext:
    """Records the constructor arguments and every solve; each solve returns the next scripted
    status for all right-hand sides (the last one repeats)."""
    instances = []
    script = [0]

    def __init__(self, dims, mass, csw_r, csw_t=None, **kw):
        self.args = dict(dims=tuple(dims), mass=mass, csw_r=csw_r, csw_t=csw_t, **kw)
        self.solves = []
        self.gauge = None
        FakeContext.instances.append(self)

    def load_gauge(self, links):
        self.gauge = links

    def load_precond(self, path):
        self.precond = path

    def solve(self, chi, **kw):
        chi = np.asarray(chi)
        n = 1 if chi.ndim == 2 else chi.shape[0]
        status = FakeContext.script[min(len(self.solves), len(FakeContext.script) - 1)]
        self.solves.append(kw)
        rel = 1e-11 if status == 0 else 1e-3
        res = [{"n_count": 10 + len(self.solves), "resid": rel, "rel_resid": rel, "status": status, "seconds": 0.0}
               for _ in range(n)]
        out = np.full(chi.shape, len(self.solves), dtype=np.complex128)
        return out, res, status


@pytest.fixture
def fake(monkeypatch):
    FakeContext.instances = []
    FakeContext.script = [0]
    monkeypatch.setattr(SS.G, "Context", FakeContext)
    return FakeContext


def _xml(silent=False, backup=False):
    return XML.format(silent="<SilentFail>true</SilentFail>" if silent else "", backup=BACKUP if backup else "")


def _solver(xml, kind="linop", operator="EOPREC_CLOVER"):
    links = np.zeros((V, 4, 3, 3), dtype=np.complex128)
    f = SS.TheLinOpFermSystemSolverFactory if kind == "linop" else SS.TheMdagMFermSystemSolverFactory
    return f.createObject("GB300_CLOVER_INVERTER", xml, ".", links, DIMS, operator=operator)


def _chi(n=None):
    shape = (V, 12) if n is None else (n, V, 12)
    return np.ones(shape, dtype=np.complex128)


def test_context_gets_the_action(fake):
    s = _solver(_xml())
    a = fake.instances[0].args
    assert a["dims"] == DIMS and abs(a["mass"] - (1 / 0.23 - 4)) < 1e-15
    assert a["csw_r"] == 1.1 and a["csw_t"] == 0.9
    assert a["aniso"] == {"xi_0": 2.0, "nu": 0.95, "t_dir": 3}
    assert a["t_boundary"] == -1 and a["sloppy_precision"] == G.PREC_HALF
    assert fake.instances[0].gauge is not None and s.subset() == 1


def test_converged_solve(fake):
    s = _solver(_xml())
    psi, r = s(np.zeros((V, 12), dtype=np.complex128), _chi())
    kw = fake.instances[0].solves[0]
    assert kw["solver"] == G.SOLVER_BICGSTAB and kw["system"] == G.SYS_MEO
    assert kw["rsd_target"] == 1e-10 and kw["max_iter"] == 300 and kw["tol_factor"] == 10
    assert r.status == 0 and r.n_count == 11 and psi.shape == (V, 12)


def test_failure_aborts_without_silentfail(fake):
    fake.script = [G.ERR_NOT_CONVERGED]
    s = _solver(_xml())
    with pytest.raises(SS.SolverFailure):
        s(None, _chi())


def test_silentfail_returns_the_failed_result(fake):
    fake.script = [G.ERR_NOT_CONVERGED]
    s = _solver(_xml(silent=True))
    psi, r = s(None, _chi())
    assert r.status == G.ERR_NOT_CONVERGED and r.rel_resid == 1e-3


def test_backup_solver_runs_on_failure(fake):
    fake.script = [G.ERR_NOT_CONVERGED, 0]
    s = _solver(_xml(backup=True))
    psi, r = s(None, _chi())
    solves = fake.instances[0].solves
    assert len(fake.instances) == 1 and len(solves) == 2  # same context, same clover action
    assert solves[0]["solver"] == G.SOLVER_BICGSTAB
    assert solves[1]["solver"] == G.SOLVER_CG and solves[1]["max_iter"] == 9000
    assert solves[1]["rsd_target"] == 1e-11 and solves[1]["sloppy_precision"] == G.PREC_DOUBLE
    assert r.status == 0 and np.all(psi == 2)  # the backup's solution
    assert r.n_count == 11 + 12  # both solves' iterations
    # the solver's own parameters are back in place for the next call
    assert s.params.SolverType == "BICGSTAB" and s.params.CloverParams.clovCoeffR == 1.1


def test_backup_failure_still_aborts(fake):
    fake.script = [G.ERR_NOT_CONVERGED]
    s = _solver(_xml(backup=True))
    with pytest.raises(SS.SolverFailure):
        s(None, _chi())


def test_mdagm_runs_no_backup(fake):
    # the MdagM solver has no backup (the backup group names a LinOp solver)
    fake.script = [G.ERR_NOT_CONVERGED, 0]
    s = _solver(_xml(backup=True), kind="mdagm")
    with pytest.raises(SS.SolverFailure):
        s(None, _chi())
    assert len(fake.instances[0].solves) == 1


def test_mdagm_predictor_gives_the_guess(fake):
    s = _solver(_xml(), kind="mdagm")
    guess = np.full((V, 12), 0.5, dtype=np.complex128)
    seen = {}

    def predictor(psi, chi):
        seen["called"] = True
        return guess

    s(np.zeros((V, 12), dtype=np.complex128), _chi(), predictor=predictor)
    kw = fake.instances[0].solves[0]
    assert seen and kw["system"] == G.SYS_MDAGM and kw["psi0"] is guess


@pytest.mark.parametrize("kind,system", [("linop", G.SYS_SYM), ("mdagm", G.SYS_SYM_MDAGM)])
def test_symmetric_action_selects_symmetric_system(fake, kind, system):
    s = _solver(_xml(), kind=kind, operator="SEOPREC_CLOVER")
    s(None, _chi())
    assert fake.instances[0].solves[0]["system"] == system


def test_multi_rhs_results(fake):
    s = _solver(_xml())
    psi, rs = s(None, _chi(12))
    assert psi.shape == (12, V, 12) and len(rs) == 12 and all(r.status == 0 for r in rs)



def _propagator_source(seed=3):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(V, 4, 4, 3, 3)) + 1j * rng.normal(size=(V, 4, 4, 3, 3))


@pytest.mark.parametrize("spin_type,solved", [("FULL", (0, 1, 2, 3)), ("UPPER", (0, 1)), ("LOWER", (2, 3))])
def test_quark_prop4_batches_the_sources(fake, spin_type, solved):
    """quarkProp4_a's per-source loop becomes one device call with every spin-colour source;
    the sources are normalised like quarkProp4_a's and the solutions scaled back and placed by
    (spin, colour), with UPPER / LOWER filling the other columns by negated copies."""
    qprop = SS.PrecFermActQprop(np.zeros((V, 4, 3, 3), complex), DIMS,
                                SS.SysSolverGB300CloverParams.from_xml(XML.format(silent="", backup="")))
    q_src = _propagator_source()
    q_sol, ncg, results = SS.quark_prop4(qprop, q_src, spin_type)
    ctx = FakeContext.instances[-1]
    assert len(ctx.solves) == 1  # one batched call, not one per source
    assert ctx.solves[0]["system"] == G.SYS_FULL
    n = 3 * len(solved)
    assert len(results) == n and ncg == sum(r.n_count for r in results)
    # the scripted solve returns psi = 1 for the unit-norm source: the solution is |chi| everywhere
    for c in range(3):
        for s in solved:
            nrm = np.linalg.norm(q_src[:, :, s, :, c])
            assert np.allclose(q_sol[:, :, s, :, c], nrm)
    for c in range(3):
        for s in set(range(4)) - set(solved):
            other = s - 2 if spin_type == "UPPER" else s + 2
            assert np.allclose(q_sol[:, :, s, :, c], -q_sol[:, :, other, :, c])
