"""Chroma-shaped host interface of the GB300 clover solver.

Mirrors, for Python callers and for the tests, the interface that the C++ adapter in
``chroma_plugin/`` gives Chroma:

- ``SysSolverGB300CloverParams``: the QUDA clover XML schema (syssolver_quda_clover_params.cc:12-131)
  plus optional tags (SolverType MIXED/FGMRES/BICGSTAB, NKrylov, NDefl, PrecondWeights, InnerTol);
  QUDA's GCR maps to FGMRES (both minimise the residual over a flexible Krylov space);
- ``TheLinOpFermSystemSolverFactory`` / ``TheMdagMFermSystemSolverFactory``: string-keyed
  factories (syssolver_linop_factory.h:29-39, syssolver_mdagm_factory.h:28-39) with the entry
  ``GB300_CLOVER_INVERTER``;
- ``LinOpSysSolverGB300Clover``: ``__call__(psi, chi) -> SystemSolverResults_t`` solving
  M~ psi_o = chi_o on the odd sites (syssolver_linop.h, eoprec_clover_linop_w.cc:142-187);
- ``MdagMSysSolverGB300Clover``: M~^dag M~ psi = chi (syssolver_mdagm.h:25-35);
- ``PrecFermActQprop``: the full-lattice propagator solve (eoprec_fermact_qprop.cc:41-80);
- ``quark_prop4``: the spin-colour sources of a propagator solved as one batch, in place of
  quarkProp4_a's per-source loop (quarkprop4_w.cc:31-175).
Failure handling follows syssolver_linop_clover_quda_w.h:636-643: a relative residual above
RsdToleranceFactor * RsdTarget raises ``SolverFailure`` unless SilentFail is set, and a
BackupSolverParam group runs the backup solver instead (Chroma's QUDA clover solver reads that
group, syssolver_quda_clover_params.cc:105-115, but never runs it).
"""
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import gbclover as G

_PREC = {"HALF": G.PREC_HALF, "SINGLE": G.PREC_SINGLE, "DOUBLE": G.PREC_DOUBLE}
_RECON = {"RECONS_12": G.RECON_12, "RECONS_NONE": G.RECON_18, "RECONS_18": G.RECON_18, "RECONS_8": G.RECON_12}
_SOLVER = {"CG": G.SOLVER_CG, "RELIABLE_CG": G.SOLVER_RELIABLE_CG, "MIXED": G.SOLVER_MIXED,
           "BICGSTAB": G.SOLVER_BICGSTAB, "GCR": G.SOLVER_FGMRES, "FGMRES": G.SOLVER_FGMRES}


class SolverFailure(RuntimeError):
    pass


@dataclass
class SystemSolverResults_t:
    """lib/syssolver.h:16-23"""
    n_count: int = 0
    resid: float = 0.0
    rel_resid: float = 0.0
    status: int = 0
    seconds: float = 0.0


def kappa_to_mass(kappa):
    """lib/io/param_io.cc:12-15: Mass = 1/(2 Kappa) - Nd."""
    return 1.0 / (2.0 * kappa) - 4.0


@dataclass
class CloverFermActParams:
    """clover_fermact_params_w.cc:27-99 (Mass | Kappa, clovCoeff | clovCoeffR/T + AnisoParam, TwistedM)."""
    Mass: float = 0.0
    clovCoeffR: float = 0.0
    clovCoeffT: float = 0.0
    u0: float = 1.0
    anisoP: bool = False
    t_dir: int = 3
    xi_0: float = 1.0
    nu: float = 1.0
    twisted_m: float = None

    @classmethod
    def from_xml(cls, node):
        p = cls()
        mass = node.find("Mass")
        kappa = node.find("Kappa")
        if mass is not None and kappa is not None:
            raise ValueError("found both a Kappa and a Mass tag")
        if mass is not None:
            p.Mass = float(mass.text)
        elif kappa is not None:
            p.Mass = kappa_to_mass(float(kappa.text))
        else:
            raise ValueError("neither Mass or Kappa found")
        if node.find("u0") is not None:
            p.u0 = float(node.find("u0").text)
        an = node.find("AnisoParam")
        if an is not None:
            p.anisoP = an.findtext("anisoP", "false").strip().lower() == "true"
            p.t_dir = int(an.findtext("t_dir", "3"))
            p.xi_0 = float(an.findtext("xi_0", "1"))
            p.nu = float(an.findtext("nu", "1"))
        if p.anisoP:
            p.clovCoeffR = float(node.findtext("clovCoeffR"))
            p.clovCoeffT = float(node.findtext("clovCoeffT"))
        else:
            p.clovCoeffR = p.clovCoeffT = float(node.findtext("clovCoeff"))
        if node.find("TwistedM") is not None:
            p.twisted_m = float(node.findtext("TwistedM"))
        return p


@dataclass
class SysSolverGB300CloverParams:
    """SysSolverQUDACloverParams fields (syssolver_quda_clover_params.h:15-90) + GB300 options."""
    MaxIter: int = 10000
    RsdTarget: float = 1e-10
    CloverParams: CloverFermActParams = field(default_factory=CloverFermActParams)
    AntiPeriodicT: bool = True
    Delta: float = 0.1
    SolverType: str = "MIXED"
    CudaPrecision: str = "DOUBLE"
    CudaSloppyPrecision: str = "HALF"
    CudaReconstruct: str = "RECONS_NONE"
    CudaSloppyReconstruct: str = "RECONS_12"
    RsdToleranceFactor: float = 10.0
    SilentFail: bool = False
    BackupSolverParam: str = None
    Verbose: bool = False
    NKrylov: int = 16
    NDefl: int = 0
    PrecondWeights: str = None
    InnerTol: float = 1e-6

    @classmethod
    def from_xml(cls, xml, path="."):
        root = ET.fromstring(xml) if isinstance(xml, str) else xml
        node = root if path in (".", "", None) else root.find(path)
        p = cls()
        p.MaxIter = int(node.findtext("MaxIter", "10000"))
        p.RsdTarget = float(node.findtext("RsdTarget", "1e-10"))
        p.CloverParams = CloverFermActParams.from_xml(node.find("CloverParams"))
        p.AntiPeriodicT = node.findtext("AntiPeriodicT", "true").strip().lower() == "true"
        p.Delta = float(node.findtext("Delta", "0.1"))
        p.SolverType = node.findtext("SolverType", "MIXED").strip()
        if p.SolverType not in _SOLVER:
            raise ValueError(f"unknown SolverType {p.SolverType}")
        for tag in ("CudaPrecision", "CudaSloppyPrecision", "CudaReconstruct", "CudaSloppyReconstruct"):
            if node.find(tag) is not None:
                setattr(p, tag, node.findtext(tag).strip())
        p.RsdToleranceFactor = float(node.findtext("RsdToleranceFactor", "10"))
        p.SilentFail = node.findtext("SilentFail", "false").strip().lower() == "true"
        bk = node.find("BackupSolverParam")
        p.BackupSolverParam = ET.tostring(bk, encoding="unicode") if bk is not None else None
        p.Verbose = node.findtext("Verbose", "false").strip().lower() == "true"
        p.NKrylov = int(node.findtext("NKrylov", "16"))
        p.NDefl = int(node.findtext("NDefl", "0"))
        p.PrecondWeights = node.findtext("PrecondWeights")
        p.InnerTol = float(node.findtext("InnerTol", "1e-6"))
        return p


class _Base:
    system = G.SYS_MEO
    symmetric_system = None
    runs_backup = True  # the LinOp solvers run BackupSolverParam; the MdagM solver does not

    def __init__(self, links, dims, params: SysSolverGB300CloverParams, max_rhs=12, operator="EOPREC_CLOVER"):
        """operator: the FermAct whose LinearOperator the solver inverts; "SEOPREC_CLOVER" selects the
        symmetric operator M_s (SymEvenOddPrecCloverLinOp) instead of M~ (EvenOddPrecCloverLinOp)."""
        if operator == "SEOPREC_CLOVER":
            if self.symmetric_system is None:
                raise ValueError(f"{type(self).__name__} has no symmetric form")
            self.system = self.symmetric_system
        elif operator != "EOPREC_CLOVER":
            raise ValueError(f"unsupported operator {operator}")
        self.params = params
        cp = params.CloverParams
        aniso = {"xi_0": cp.xi_0, "nu": cp.nu, "t_dir": cp.t_dir} if cp.anisoP else None
        self.ctx = G.Context(dims, cp.Mass, cp.clovCoeffR, cp.clovCoeffT,
                             t_boundary=-1 if params.AntiPeriodicT else 1,
                             sloppy_precision=_PREC[params.CudaSloppyPrecision],
                             sloppy_reconstruct=_RECON[params.CudaSloppyReconstruct], max_rhs=max_rhs, aniso=aniso,
                             twisted_m=cp.twisted_m, verbose=params.Verbose)
        self.ctx.load_gauge(links)
        if params.PrecondWeights:
            self.ctx.load_precond(params.PrecondWeights)
        self.dims = tuple(dims)

    def subset(self):
        """rb[1]: the odd checkerboard (EvenOddPrecLinearOperator::subset, eoprec_linop.h:98)."""
        return 1

    def _solve(self, psi, chi):
        p = self.params
        multi = np.asarray(chi).ndim == 3 or (np.asarray(chi).ndim == 2 and np.asarray(chi).shape[-1] != 12)
        out, res, rc = self.ctx.solve(chi, solver=_SOLVER[p.SolverType], system=self.system, rsd_target=p.RsdTarget,
                                      max_iter=p.MaxIter, delta=p.Delta,
                                      sloppy_precision=_PREC[p.CudaSloppyPrecision], inner_tol=p.InnerTol,
                                      nkrylov=p.NKrylov, ndefl=p.NDefl, use_precond=int(bool(p.PrecondWeights)),
                                      psi0=psi,
                                      tol_factor=p.RsdToleranceFactor, raise_on_error=False)
        results = [SystemSolverResults_t(r["n_count"], r["resid"], r["rel_resid"], r["status"], r["seconds"])
                   for r in res]
        bad = [r for r in results if r.status != 0]
        if bad:
            if p.BackupSolverParam and self.runs_backup:
                # the backup solves the same system on this context; its iterations add to the
                # failed solve's, as in the C++ adapter
                backup = SysSolverGB300CloverParams.from_xml(p.BackupSolverParam)
                backup.CloverParams = p.CloverParams
                saved, self.params = self.params, backup
                try:
                    psi_out, res2 = self._solve(psi, chi)
                finally:
                    self.params = saved
                for a, b in zip(res2 if multi else [res2], results):
                    a.n_count += b.n_count
                return psi_out, res2
            if not p.SilentFail:
                raise SolverFailure(f"GB300_CLOVER_INVERTER failed: {bad[0]}")
        psi_out = out.reshape(np.asarray(chi).shape)
        return psi_out, (results if multi else results[0])


class LinOpSysSolverGB300Clover(_Base):
    """LinOpSystemSolver<LatticeFermion>: M~ psi_o = chi_o (only rb[1] of psi/chi meaningful), or
    M_s psi_o = chi_o for a SEOPREC_CLOVER action."""
    system = G.SYS_MEO
    symmetric_system = G.SYS_SYM

    def __call__(self, psi, chi):
        return self._solve(psi, chi)


class MdagMSysSolverGB300Clover(_Base):
    """MdagMSystemSolver<LatticeFermion>: M~^dag M~ psi = chi (chronological predictor: psi guess), or
    M_s^dag M_s psi = chi for a SEOPREC_CLOVER action."""
    system = G.SYS_MDAGM
    symmetric_system = G.SYS_SYM_MDAGM
    runs_backup = False

    def __call__(self, psi, chi, predictor=None):
        if predictor is not None:
            psi = predictor(psi, chi)
        return self._solve(psi, chi)


class PrecFermActQprop(_Base):
    """Full-lattice solve M psi = chi: Schur prep, odd solve, even reconstruction, full residual."""
    system = G.SYS_FULL

    def __call__(self, psi, chi):
        return self._solve(psi, chi)


_SPIN_RANGE = {"FULL": (0, 4), "UPPER": (0, 2), "LOWER": (2, 4)}


def quark_prop4(qprop, q_src, quark_spin_type="FULL"):
    """The batched counterpart of Chroma's quarkProp4_a (lib/actions/ferm/qprop/quarkprop4_w.cc:31-175)
    for a GB300 full-system solver (``PrecFermActQprop``), as chroma_plugin's quarkProp4GB300.

    quarkProp4_a calls the factory solver once per spin-colour source; here the sources are
    extracted in its order (colour outer, spin inner; PropToFerm), each scaled to unit norm as it
    does, and solved together as one multi-right-hand-side batch, then scaled back and placed in
    the solution propagator (FermToProp).  QUARK_SPIN_TYPE_UPPER / _LOWER solve half the spin
    columns and fill the other half with their negated copies (quarkprop4_w.cc:120-175).

    q_src: complex array (V, Ns, Ns, Nc, Nc) indexed [site, sink spin, source spin, sink colour,
    source colour], QDP++'s prop.elem(site).elem(s1, s2).elem(c1, c2).
    Returns (q_sol, ncg_had, per-source SystemSolverResults_t)."""
    q_src = np.asarray(q_src, dtype=np.complex128)
    V = q_src.shape[0]
    start, end = _SPIN_RANGE[quark_spin_type]
    cols = [(c, s) for c in range(3) for s in range(start, end)]
    chi = np.ascontiguousarray(np.stack([q_src[:, :, s, :, c] for c, s in cols]).reshape(len(cols), V, 12))
    nrm = np.sqrt(np.einsum("kvi,kvi->k", chi.conj(), chi).real)
    fact = np.where(nrm != 0.0, 1.0 / np.where(nrm != 0.0, nrm, 1.0), 1.0)
    chi *= fact[:, None, None]
    psi, results = qprop(None, chi)
    results = results if isinstance(results, list) else [results]
    q_sol = np.zeros_like(q_src)
    for k, (c, s) in enumerate(cols):
        sol = (psi[k] / fact[k]).reshape(V, 4, 3)
        q_sol[:, :, s, :, c] = sol
        if quark_spin_type == "UPPER":
            q_sol[:, :, s + 2, :, c] = -sol
        elif quark_spin_type == "LOWER":
            q_sol[:, :, s - 2, :, c] = -sol
    return q_sol, int(sum(r.n_count for r in results)), results


class _Factory:
    def __init__(self):
        self._creators = {}

    def registerObject(self, name, creator):
        if name in self._creators:
            return False
        self._creators[name] = creator
        return True

    def createObject(self, name, xml, path, links, dims, operator="EOPREC_CLOVER"):
        if name not in self._creators:
            # objfactory.h:44-53 throws a string on an unknown key
            raise KeyError(f"Factory error: unknown id {name}")
        return self._creators[name](xml, path, links, dims, operator)

    def keys(self):
        return sorted(self._creators)


TheLinOpFermSystemSolverFactory = _Factory()
TheMdagMFermSystemSolverFactory = _Factory()
TheLinOpFermSystemSolverFactory.registerObject(
    "GB300_CLOVER_INVERTER",
    lambda xml, path, links, dims, operator="EOPREC_CLOVER": LinOpSysSolverGB300Clover(
        links, dims, SysSolverGB300CloverParams.from_xml(xml, path), operator=operator))
TheMdagMFermSystemSolverFactory.registerObject(
    "GB300_CLOVER_INVERTER",
    lambda xml, path, links, dims, operator="EOPREC_CLOVER": MdagMSysSolverGB300Clover(
        links, dims, SysSolverGB300CloverParams.from_xml(xml, path), operator=operator))
