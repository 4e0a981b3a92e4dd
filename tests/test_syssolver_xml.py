"""Host-side logic of the Chroma-shaped interface (no GPU): the QUDA clover XML schema
(syssolver_quda_clover_params.cc:12-131), CloverFermActParams (clover_fermact_params_w.cc:27-99)
and the string-keyed factories (objfactory.h:44-135)."""
import numpy as np
import pytest

from chroma_gb300 import syssolver as SS

QUDA_XML = """
<InvertParam>
  <invType>GB300_CLOVER_INVERTER</invType>
  <CloverParams>
    <Kappa>0.1250</Kappa>
    <clovCoeff>1.6</clovCoeff>
  </CloverParams>
  <RsdTarget>1e-10</RsdTarget>
  <MaxIter>5000</MaxIter>
  <AntiPeriodicT>true</AntiPeriodicT>
  <Delta>0.05</Delta>
  <SolverType>CG</SolverType>
  <CudaPrecision>DOUBLE</CudaPrecision>
  <CudaSloppyPrecision>SINGLE</CudaSloppyPrecision>
  <CudaReconstruct>RECONS_NONE</CudaReconstruct>
  <CudaSloppyReconstruct>RECONS_12</CudaSloppyReconstruct>
  <AsymmetricLinop>false</AsymmetricLinop>
  <AutotuneDslash>true</AutotuneDslash>
  <RsdToleranceFactor>50</RsdToleranceFactor>
  <SilentFail>true</SilentFail>
  <BackupSolverParam>
    <invType>GB300_CLOVER_INVERTER</invType>
    <CloverParams><Kappa>0.1250</Kappa><clovCoeff>1.6</clovCoeff></CloverParams>
    <RsdTarget>1e-10</RsdTarget><MaxIter>20000</MaxIter><AntiPeriodicT>true</AntiPeriodicT>
    <SolverType>CG</SolverType>
  </BackupSolverParam>
</InvertParam>
"""


def test_quda_schema_parses():
    p = SS.SysSolverGB300CloverParams.from_xml(QUDA_XML)
    assert p.MaxIter == 5000 and p.RsdTarget == 1e-10 and p.Delta == 0.05
    assert p.SolverType == "CG" and p.CudaSloppyPrecision == "SINGLE"
    assert p.RsdToleranceFactor == 50 and p.SilentFail is True
    assert abs(p.CloverParams.Mass - (1 / (2 * 0.125) - 4)) < 1e-15
    assert p.CloverParams.clovCoeffR == p.CloverParams.clovCoeffT == 1.6
    assert p.BackupSolverParam is not None
    b = SS.SysSolverGB300CloverParams.from_xml(p.BackupSolverParam)
    assert b.MaxIter == 20000


def test_kappa_and_mass_conflict():
    bad = QUDA_XML.replace("<Kappa>0.1250</Kappa>\n", "<Kappa>0.1250</Kappa><Mass>0.1</Mass>\n", 1)
    with pytest.raises(ValueError):
        SS.SysSolverGB300CloverParams.from_xml(bad)


def test_aniso_params():
    xml = """<P><CloverParams><Mass>0.1</Mass><clovCoeffR>1.2</clovCoeffR><clovCoeffT>0.9</clovCoeffT>
             <AnisoParam><anisoP>true</anisoP><t_dir>3</t_dir><xi_0>2.0</xi_0><nu>0.9</nu></AnisoParam>
             </CloverParams><RsdTarget>1e-8</RsdTarget><MaxIter>10</MaxIter><AntiPeriodicT>false</AntiPeriodicT></P>"""
    p = SS.SysSolverGB300CloverParams.from_xml(xml)
    cp = p.CloverParams
    assert cp.anisoP and cp.xi_0 == 2.0 and cp.nu == 0.9 and cp.clovCoeffR == 1.2 and cp.clovCoeffT == 0.9
    assert p.AntiPeriodicT is False


def test_factories():
    assert "GB300_CLOVER_INVERTER" in SS.TheLinOpFermSystemSolverFactory.keys()
    assert "GB300_CLOVER_INVERTER" in SS.TheMdagMFermSystemSolverFactory.keys()
    assert not SS.TheLinOpFermSystemSolverFactory.registerObject("GB300_CLOVER_INVERTER", lambda *a: None)
    with pytest.raises(KeyError):
        SS.TheLinOpFermSystemSolverFactory.createObject("NOPE", QUDA_XML, ".", None, None)
    # an operator the solver does not invert is refused before any device work
    with pytest.raises(ValueError):
        SS.TheLinOpFermSystemSolverFactory.createObject("GB300_CLOVER_INVERTER", QUDA_XML, ".", None, None,
                                                        operator="UNPRECONDITIONED_WILSON")
    with pytest.raises(ValueError):
        SS.PrecFermActQprop(None, None, SS.SysSolverGB300CloverParams.from_xml(QUDA_XML), operator="SEOPREC_CLOVER")


def test_unknown_solver_type():
    with pytest.raises(ValueError):
        SS.SysSolverGB300CloverParams.from_xml(QUDA_XML.replace("<SolverType>CG", "<SolverType>NOPE", 1))


def test_kappa_to_mass():
    assert SS.kappa_to_mass(0.125) == 0.0
    assert np.isclose(SS.kappa_to_mass(0.115), 1 / 0.23 - 4)


@pytest.mark.parametrize("name,code", [("CG", "SOLVER_CG"), ("RELIABLE_CG", "SOLVER_RELIABLE_CG"),
                                       ("MIXED", "SOLVER_MIXED"), ("BICGSTAB", "SOLVER_BICGSTAB"),
                                       ("GCR", "SOLVER_FGMRES"), ("FGMRES", "SOLVER_FGMRES")])
def test_solver_type_map(name, code):
    """QUDA's SolverType strings select the library solver: BICGSTAB the inner reliable BiCGStab,
    GCR the flexible-Krylov FGMRES (both minimise over a flexible space)."""
    from chroma_gb300 import gbclover as G
    p = SS.SysSolverGB300CloverParams.from_xml(QUDA_XML.replace("<SolverType>CG", f"<SolverType>{name}", 1))
    assert p.SolverType == name
    assert SS._SOLVER[name] == getattr(G, code)
