// -*- C++ -*-
/*! \file
 *  \brief Parameters of GB300_CLOVER_INVERTER: the QUDA clover schema plus the GB300 options.
 *
 *  The XML layout is the one of SysSolverQUDACloverParams
 *  (lib/actions/ferm/invert/quda_solvers/syssolver_quda_clover_params.{h:15-90,cc:12-131}), so an
 *  existing QUDA_CLOVER_INVERTER input runs after changing <invType> only.  Optional tags:
 *  SolverType MIXED | BICGSTAB | FGMRES | GCR | RELIABLE_CG | CG, NKrylov, NDefl, InnerTol, PrecondWeights,
 *  MaxRHS.
 *  Compiled only inside a Chroma build (needs QDP++).
 */
#ifndef __syssolver_gb300_clover_params_h__
#define __syssolver_gb300_clover_params_h__

#include <string>

#include "chromabase.h"
#include "actions/ferm/fermacts/clover_fermact_params_w.h"
#include "io/xml_group_reader.h"

namespace Chroma
{
  struct SysSolverGB300CloverParams
  {
    SysSolverGB300CloverParams(XMLReader& xml, const std::string& path);
    SysSolverGB300CloverParams();

    int MaxIter;
    Real RsdTarget;
    CloverFermActParams CloverParams;
    bool AntiPeriodicT;
    Real Delta;
    std::string SolverType;           // CG | RELIABLE_CG | MIXED | BICGSTAB | FGMRES (GCR -> FGMRES)
    std::string CudaSloppyPrecision;  // HALF | SINGLE | DOUBLE
    std::string CudaSloppyReconstruct;// RECONS_12 | RECONS_NONE
    Real RsdToleranceFactor;
    bool SilentFail;
    bool backup_invP;
    GroupXML_t backup_inv_param;
    bool verboseP;
    int NKrylov;
    int NDefl;  //!< FGMRES-DR deflation space (FGMRESDR_INVERTER's NDefl)
    Real InnerTol;
    std::string PrecondWeights;       // empty: no learned preconditioner
    int MaxRHS;
  };

  void read(XMLReader& xml, const std::string& path, SysSolverGB300CloverParams& p);
  void write(XMLWriter& xml, const std::string& path, const SysSolverGB300CloverParams& p);

}  // namespace Chroma

#endif
