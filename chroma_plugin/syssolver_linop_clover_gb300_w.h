// -*- C++ -*-
/*! \file
 *  \brief GB300_CLOVER_INVERTER: the even-odd clover solve on one GB300 through libgbclover.
 *
 *  Drop-in for the LinOp factory (lib/actions/ferm/invert/syssolver_linop_factory.h:29-39) and
 *  the MdagM factory (syssolver_mdagm_factory.h:28-39), shaped after LinOpSysSolverQUDAClover
 *  (quda_solvers/syssolver_linop_clover_quda_w.h:50-643).  The constructor gathers the
 *  BC-modified (and possibly smeared) links of the FermState by lattice coordinate and hands
 *  them to the device, which builds the clover term and its even-parity inverse itself.
 *  Compiled only inside a Chroma build (needs QDP++).
 */
#ifndef __syssolver_linop_clover_gb300_w_h__
#define __syssolver_linop_clover_gb300_w_h__

#include <vector>

#include "chromabase.h"
#include "handle.h"
#include "linearop.h"
#include "state.h"
#include "syssolver.h"
#include "actions/ferm/invert/syssolver_linop.h"
#include "actions/ferm/invert/syssolver_mdagm.h"
#include "chroma_plugin/syssolver_gb300_clover_params.h"
#include "gbclover.h"

namespace Chroma
{
  namespace LinOpSysSolverGB300CloverEnv { bool registerAll(); }
  namespace MdagMSysSolverGB300CloverEnv { bool registerAll(); }

  //! Device context shared by the LinOp and MdagM solvers of one FermState
  class GB300CloverContext
  {
  public:
    typedef multi1d<LatticeColorMatrix> Q;
    GB300CloverContext(Handle<FermState<LatticeFermion, Q, Q> > state, const SysSolverGB300CloverParams& p);
    ~GB300CloverContext();
    gbc_ctx* get() const { return ctx; }
    //! full-lattice LatticeFermion <-> canonical host buffer (x fastest, [spin][colour])
    void gather(std::vector<double>& buf, const LatticeFermion& f) const;
    void scatter(LatticeFermion& f, const std::vector<double>& buf, int parity_mask) const;
  private:
    gbc_ctx* ctx;
  };

  //! GBC_SYS_SYM* when A is the symmetric operator of a SEOPREC_CLOVER action
  //! (SymEvenOddPrecCloverLinOp, seoprec_clover_linop_w.h), else the asymmetric systems
  bool is_symmetric_clover(const Handle<LinearOperator<LatticeFermion> >& A);

  //! Solves M~ psi_o = chi_o (only rb[1] meaningful), M~ = A_oo - 1/4 D_oe A_ee^-1 D_eo, or
  //! M_s psi_o = chi_o, M_s = 1 - 1/4 A_oo^-1 D_oe A_ee^-1 D_eo, for a symmetric operator A
  class LinOpSysSolverGB300Clover : public LinOpSystemSolver<LatticeFermion>
  {
  public:
    typedef LatticeFermion T;
    typedef multi1d<LatticeColorMatrix> Q;
    LinOpSysSolverGB300Clover(Handle<LinearOperator<T> > A_, Handle<FermState<T, Q, Q> > state_,
                              const SysSolverGB300CloverParams& p);
    ~LinOpSysSolverGB300Clover() {}
    const Subset& subset() const { return A->subset(); }
    SystemSolverResults_t operator()(T& psi, const T& chi) const;
  private:
    Handle<LinearOperator<T> > A;
    Handle<FermState<T, Q, Q> > state;
    SysSolverGB300CloverParams invParam;
    Handle<GB300CloverContext> dev;
    int system;
  };

  //! Solves M~^dag M~ psi = chi (HMC; M_s^dag M_s for a symmetric A), with the chronological
  //! predictor as initial guess
  class MdagMSysSolverGB300Clover : public MdagMSystemSolver<LatticeFermion>
  {
  public:
    typedef LatticeFermion T;
    typedef multi1d<LatticeColorMatrix> Q;
    MdagMSysSolverGB300Clover(Handle<LinearOperator<T> > A_, Handle<FermState<T, Q, Q> > state_,
                              const SysSolverGB300CloverParams& p);
    ~MdagMSysSolverGB300Clover() {}
    const Subset& subset() const { return A->subset(); }
    SystemSolverResults_t operator()(T& psi, const T& chi) const;
    SystemSolverResults_t operator()(T& psi, const T& chi, AbsChronologicalPredictor4D<T>& predictor) const;
  private:
    Handle<LinearOperator<T> > A;
    Handle<FermState<T, Q, Q> > state;
    SysSolverGB300CloverParams invParam;
    Handle<GB300CloverContext> dev;
    int system;
  };

}  // namespace Chroma

#endif
