/*! \file
 *  \brief Reader/writer of the GB300_CLOVER_INVERTER parameters (QUDA clover schema + options).
 */
#include "chroma_plugin/syssolver_gb300_clover_params.h"

namespace Chroma
{
  SysSolverGB300CloverParams::SysSolverGB300CloverParams()
    : MaxIter(10000), RsdTarget(1.0e-10), AntiPeriodicT(true), Delta(0.1), SolverType("MIXED"),
      CudaSloppyPrecision("HALF"), CudaSloppyReconstruct("RECONS_12"), RsdToleranceFactor(10),
      SilentFail(false), backup_invP(false), verboseP(false), NKrylov(16), NDefl(0), InnerTol(1.0e-6), MaxRHS(12)
  {}

  SysSolverGB300CloverParams::SysSolverGB300CloverParams(XMLReader& xml, const std::string& path)
    : SysSolverGB300CloverParams()
  {
    XMLReader paramtop(xml, path);
    read(paramtop, "MaxIter", MaxIter);
    read(paramtop, "RsdTarget", RsdTarget);
    read(paramtop, "CloverParams", CloverParams);
    read(paramtop, "AntiPeriodicT", AntiPeriodicT);
    if (paramtop.count("Delta") > 0) read(paramtop, "Delta", Delta);
    if (paramtop.count("SolverType") > 0) read(paramtop, "SolverType", SolverType);
    if (paramtop.count("CudaSloppyPrecision") > 0) read(paramtop, "CudaSloppyPrecision", CudaSloppyPrecision);
    if (paramtop.count("CudaSloppyReconstruct") > 0)
      read(paramtop, "CudaSloppyReconstruct", CudaSloppyReconstruct);
    if (paramtop.count("RsdToleranceFactor") > 0) read(paramtop, "RsdToleranceFactor", RsdToleranceFactor);
    if (paramtop.count("SilentFail") > 0) read(paramtop, "SilentFail", SilentFail);
    if (paramtop.count("BackupSolverParam") > 0) {
      backup_invP = true;
      backup_inv_param = readXMLGroup(paramtop, "BackupSolverParam", "invType");
    }
    if (paramtop.count("Verbose") > 0) read(paramtop, "Verbose", verboseP);
    if (paramtop.count("NKrylov") > 0) read(paramtop, "NKrylov", NKrylov);
    if (paramtop.count("NDefl") > 0) read(paramtop, "NDefl", NDefl);
    if (paramtop.count("InnerTol") > 0) read(paramtop, "InnerTol", InnerTol);
    if (paramtop.count("PrecondWeights") > 0) read(paramtop, "PrecondWeights", PrecondWeights);
    if (paramtop.count("MaxRHS") > 0) read(paramtop, "MaxRHS", MaxRHS);
    // The QUDA-only tags (CudaPrecision, CudaReconstruct, AsymmetricLinop, AutotuneDslash,
    // Pipeline, GCRInnerParams, ...) are accepted and ignored: the outer precision is always
    // FP64 and the stencil shapes are autotuned.
  }

  void read(XMLReader& xml, const std::string& path, SysSolverGB300CloverParams& p)
  {
    SysSolverGB300CloverParams tmp(xml, path);
    p = tmp;
  }

  void write(XMLWriter& xml, const std::string& path, const SysSolverGB300CloverParams& p)
  {
    push(xml, path);
    write(xml, "invType", std::string("GB300_CLOVER_INVERTER"));
    write(xml, "MaxIter", p.MaxIter);
    write(xml, "RsdTarget", p.RsdTarget);
    write(xml, "CloverParams", p.CloverParams);
    write(xml, "AntiPeriodicT", p.AntiPeriodicT);
    write(xml, "Delta", p.Delta);
    write(xml, "SolverType", p.SolverType);
    write(xml, "CudaSloppyPrecision", p.CudaSloppyPrecision);
    write(xml, "CudaSloppyReconstruct", p.CudaSloppyReconstruct);
    write(xml, "RsdToleranceFactor", p.RsdToleranceFactor);
    write(xml, "SilentFail", p.SilentFail);
    write(xml, "NKrylov", p.NKrylov);
    write(xml, "NDefl", p.NDefl);
    write(xml, "InnerTol", p.InnerTol);
    if (!p.PrecondWeights.empty()) write(xml, "PrecondWeights", p.PrecondWeights);
    pop(xml);
  }
}  // namespace Chroma
