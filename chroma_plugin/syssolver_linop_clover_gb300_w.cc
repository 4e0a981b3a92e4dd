/*! \file
 *  \brief GB300_CLOVER_INVERTER registration and solve (Chroma side of libgbclover).
 */
#include "chroma_plugin/syssolver_linop_clover_gb300_w.h"

#include <limits>
#include <sstream>

#include "actions/ferm/invert/syssolver_linop_factory.h"
#include "actions/ferm/invert/syssolver_mdagm_factory.h"
#include "actions/ferm/linop/seoprec_clover_linop_w.h"
#include "lmdagm.h"

namespace Chroma
{
  namespace
  {
    int prec_code(const std::string& s)
    {
      if (s == "DOUBLE") return GBC_PREC_DOUBLE;
      if (s == "SINGLE") return GBC_PREC_SINGLE;
      return GBC_PREC_HALF;
    }
    int solver_code(const std::string& s)
    {
      if (s == "CG") return GBC_SOLVER_CG;
      if (s == "RELIABLE_CG") return GBC_SOLVER_RELIABLE_CG;
      if (s == "FGMRES" || s == "GCR") return GBC_SOLVER_FGMRES;  // both minimise over a flexible Krylov space
      if (s == "BICGSTAB") return GBC_SOLVER_BICGSTAB;
      return GBC_SOLVER_MIXED;
    }
    // canonical site index s = x + Lx*(y + Ly*(z + Lz*t)) -> QDP++ linear index on this node
    int qdp_index(long s)
    {
      multi1d<int> x(Nd);
      for (int m = 0; m < Nd; ++m) {
        x[m] = s % Layout::lattSize()[m];
        s /= Layout::lattSize()[m];
      }
      return Layout::linearSiteIndex(x);
    }
    gbc_solve_params make_params(const SysSolverGB300CloverParams& p, int system)
    {
      gbc_solve_params q;
      q.solver = solver_code(p.SolverType);
      q.system = system;
      q.rsd_target = toDouble(p.RsdTarget);
      q.max_iter = p.MaxIter;
      q.delta = toDouble(p.Delta);
      q.rsd_tolerance_factor = toDouble(p.RsdToleranceFactor);
      q.sloppy_precision = prec_code(p.CudaSloppyPrecision);
      q.inner_tol = toDouble(p.InnerTol);
      q.inner_max_iter = 0;
      q.nkrylov = p.NKrylov;
      q.ndefl = p.NDefl;
      q.use_precond = p.PrecondWeights.empty() ? 0 : 1;
      q.zero_guess = 0;
      return q;
    }
  }  // namespace

  GB300CloverContext::GB300CloverContext(Handle<FermState<LatticeFermion, Q, Q> > state,
                                         const SysSolverGB300CloverParams& p)
    : ctx(nullptr)
  {
    if (Layout::numNodes() != 1) {
      QDPIO::cerr << "GB300_CLOVER_INVERTER: one rank per GPU, no domain decomposition" << std::endl;
      QDP_abort(1);
    }
    gbc_geom g;
    for (int m = 0; m < Nd; ++m) g.dims[m] = Layout::lattSize()[m];
    g.t_boundary = p.AntiPeriodicT ? -1 : 1;
    const CloverFermActParams& cp = p.CloverParams;
    gbc_action a;
    a.mass = toDouble(cp.Mass);
    a.clov_coeff_r = toDouble(cp.clovCoeffR);
    a.clov_coeff_t = toDouble(cp.clovCoeffT);
    a.aniso = cp.anisoParam.anisoP ? 1 : 0;
    a.xi_0 = toDouble(cp.anisoParam.xi_0);
    a.nu = toDouble(cp.anisoParam.nu);
    a.t_dir = cp.anisoParam.t_dir;
    a.twisted = cp.twisted_m_usedP ? 1 : 0;
    a.twisted_m = toDouble(cp.twisted_m);
    gbc_opts o;
    o.sloppy_precision = prec_code(p.CudaSloppyPrecision);
    o.sloppy_reconstruct = p.CudaSloppyReconstruct == "RECONS_NONE" ? GBC_RECON_18 : GBC_RECON_12;
    o.max_rhs = p.MaxRHS;
    o.verbose = p.verboseP ? 1 : 0;
    if (gbc_create(&ctx, &g, &a, &o) != GBC_OK) {
      QDPIO::cerr << "GB300_CLOVER_INVERTER: gbc_create failed" << std::endl;
      QDP_abort(1);
    }
    // links as the solver sees them: FermState::getLinks() carries the BC and any smearing
    const Q& u = state->getLinks();
    const long V = Layout::vol();
    std::vector<double> links((size_t)V * 72);
    for (long s = 0; s < V; ++s) {
      const int lin = qdp_index(s);
      for (int mu = 0; mu < Nd; ++mu)
        for (int r = 0; r < Nc; ++r)
          for (int c = 0; c < Nc; ++c) {
            const size_t k = (((size_t)s * 4 + mu) * 9 + r * 3 + c) * 2;
            links[k] = toDouble(u[mu].elem(lin).elem().elem(r, c).real());
            links[k + 1] = toDouble(u[mu].elem(lin).elem().elem(r, c).imag());
          }
    }
    if (gbc_load_gauge(ctx, links.data()) != GBC_OK) {
      QDPIO::cerr << "GB300_CLOVER_INVERTER: " << gbc_last_error(ctx) << std::endl;
      QDP_abort(1);
    }
    if (!p.PrecondWeights.empty() && gbc_load_precond(ctx, p.PrecondWeights.c_str()) != GBC_OK) {
      QDPIO::cerr << "GB300_CLOVER_INVERTER: cannot load " << p.PrecondWeights << ": " << gbc_last_error(ctx)
                  << std::endl;
      QDP_abort(1);
    }
  }

  GB300CloverContext::~GB300CloverContext() { gbc_destroy(ctx); }

  void GB300CloverContext::gather(std::vector<double>& buf, const LatticeFermion& f) const
  {
    const long V = Layout::vol();
    buf.assign((size_t)V * 24, 0.0);
    for (long s = 0; s < V; ++s) {
      const int lin = qdp_index(s);
      for (int sp = 0; sp < Ns; ++sp)
        for (int c = 0; c < Nc; ++c) {
          const size_t k = ((size_t)s * 12 + sp * 3 + c) * 2;
          buf[k] = toDouble(f.elem(lin).elem(sp).elem(c).real());
          buf[k + 1] = toDouble(f.elem(lin).elem(sp).elem(c).imag());
        }
    }
  }

  void GB300CloverContext::scatter(LatticeFermion& f, const std::vector<double>& buf, int parity_mask) const
  {
    const long V = Layout::vol();
    for (long s = 0; s < V; ++s) {
      multi1d<int> x(Nd);
      long r = s;
      int par = 0;
      for (int m = 0; m < Nd; ++m) {
        x[m] = r % Layout::lattSize()[m];
        r /= Layout::lattSize()[m];
        par += x[m];
      }
      if (!((parity_mask >> (par & 1)) & 1)) continue;
      const int lin = Layout::linearSiteIndex(x);
      for (int sp = 0; sp < Ns; ++sp)
        for (int c = 0; c < Nc; ++c) {
          const size_t k = ((size_t)s * 12 + sp * 3 + c) * 2;
          f.elem(lin).elem(sp).elem(c).real() = buf[k];
          f.elem(lin).elem(sp).elem(c).imag() = buf[k + 1];
        }
    }
  }

  namespace
  {
    SystemSolverResults_t run(const GB300CloverContext& dev, const SysSolverGB300CloverParams& p, int system,
                              LatticeFermion& psi, const LatticeFermion& chi, bool& failed)
    {
      std::vector<double> hchi, hpsi;
      dev.gather(hchi, chi);
      dev.gather(hpsi, psi);
      gbc_solve_params q = make_params(p, system);
      // a call refused before the solve starts (bad arguments, call order, CUDA error) fills no
      // result and leaves psi as it was: report no iterations and an unknown residual then
      gbc_result r{};
      r.resid = r.rel_resid = std::numeric_limits<double>::quiet_NaN();
      int rc = gbc_solve(dev.get(), &q, 1, hpsi.data(), hchi.data(), &r);
      dev.scatter(psi, hpsi, 2);  // rb[1] only
      SystemSolverResults_t res;
      res.n_count = r.n_count;
      res.resid = r.resid;
      failed = rc != GBC_OK;
      if (failed)
        QDPIO::cerr << "GB300_CLOVER_INVERTER: " << gbc_strerror(rc) << ": " << gbc_last_error(dev.get())
                    << std::endl;
      QDPIO::cout << "GB300_CLOVER_INVERTER: " << r.n_count << " iterations (" << r.n_outer << " outer). Rsd = "
                  << r.resid << " Relative Rsd = " << r.rel_resid << " time " << r.seconds << " s" << std::endl;
      return res;
    }
  }  // namespace

  bool is_symmetric_clover(const Handle<LinearOperator<LatticeFermion> >& A)
  {
    return dynamic_cast<const SymEvenOddPrecCloverLinOp*>(A.operator->()) != nullptr;
  }

  LinOpSysSolverGB300Clover::LinOpSysSolverGB300Clover(Handle<LinearOperator<T> > A_,
                                                       Handle<FermState<T, Q, Q> > state_,
                                                       const SysSolverGB300CloverParams& p)
    : A(A_), state(state_), invParam(p), dev(new GB300CloverContext(state_, p)),
      system(is_symmetric_clover(A_) ? GBC_SYS_SYM : GBC_SYS_MEO)
  {}

  SystemSolverResults_t LinOpSysSolverGB300Clover::operator()(T& psi, const T& chi) const
  {
    START_CODE();
    bool failed = false;
    SystemSolverResults_t res = run(*dev, invParam, system, psi, chi, failed);
    if (failed) {
      // RsdToleranceFactor / SilentFail / BackupSolverParam (syssolver_linop_clover_quda_w.h:636-643)
      if (invParam.backup_invP) {
        QDPIO::cout << "GB300_CLOVER_INVERTER: running the backup solver" << std::endl;
        std::istringstream is(invParam.backup_inv_param.xml);
        XMLReader xml(is);
        Handle<LinOpSystemSolver<T> > backup(TheLinOpFermSystemSolverFactory::Instance().createObject(
            invParam.backup_inv_param.id, xml, invParam.backup_inv_param.path, state, A));
        SystemSolverResults_t r2 = (*backup)(psi, chi);
        r2.n_count += res.n_count;
        res = r2;
      } else if (!invParam.SilentFail) {
        QDPIO::cerr << "GB300_CLOVER_INVERTER: solve failed" << std::endl;
        QDP_abort(1);
      }
    }
    END_CODE();
    return res;
  }

  MdagMSysSolverGB300Clover::MdagMSysSolverGB300Clover(Handle<LinearOperator<T> > A_,
                                                       Handle<FermState<T, Q, Q> > state_,
                                                       const SysSolverGB300CloverParams& p)
    : A(A_), state(state_), invParam(p), dev(new GB300CloverContext(state_, p)),
      system(is_symmetric_clover(A_) ? GBC_SYS_SYM_MDAGM : GBC_SYS_MDAGM)
  {}

  SystemSolverResults_t MdagMSysSolverGB300Clover::operator()(T& psi, const T& chi) const
  {
    bool failed = false;
    SystemSolverResults_t res = run(*dev, invParam, system, psi, chi, failed);
    if (failed && !invParam.SilentFail) {
      QDPIO::cerr << "GB300_CLOVER_INVERTER (MdagM): solve failed" << std::endl;
      QDP_abort(1);
    }
    return res;
  }

  SystemSolverResults_t MdagMSysSolverGB300Clover::operator()(T& psi, const T& chi,
                                                              AbsChronologicalPredictor4D<T>& predictor) const
  {
    // the predictor supplies the initial guess (syssolver_mdagm_cg.h:105-125)
    Handle<LinearOperator<T> > MdagM(new MdagMLinOp<T>(A));
    predictor(psi, *MdagM, chi);
    SystemSolverResults_t res = (*this)(psi, chi);
    predictor.newVector(psi);
    return res;
  }

  namespace LinOpSysSolverGB300CloverEnv
  {
    namespace
    {
      bool registered = false;
      LinOpSystemSolver<LatticeFermion>* createFerm(
          XMLReader& xml_in, const std::string& path,
          Handle<FermState<LatticeFermion, multi1d<LatticeColorMatrix>, multi1d<LatticeColorMatrix> > > state,
          Handle<LinearOperator<LatticeFermion> > A)
      {
        return new LinOpSysSolverGB300Clover(A, state, SysSolverGB300CloverParams(xml_in, path));
      }
    }
    bool registerAll()
    {
      bool success = true;
      if (!registered) {
        success &= TheLinOpFermSystemSolverFactory::Instance().registerObject(std::string("GB300_CLOVER_INVERTER"),
                                                                               createFerm);
        registered = true;
      }
      return success;
    }
  }

  namespace MdagMSysSolverGB300CloverEnv
  {
    namespace
    {
      bool registered = false;
      MdagMSystemSolver<LatticeFermion>* createFerm(
          XMLReader& xml_in, const std::string& path,
          Handle<FermState<LatticeFermion, multi1d<LatticeColorMatrix>, multi1d<LatticeColorMatrix> > > state,
          Handle<LinearOperator<LatticeFermion> > A)
      {
        return new MdagMSysSolverGB300Clover(A, state, SysSolverGB300CloverParams(xml_in, path));
      }
    }
    bool registerAll()
    {
      bool success = true;
      if (!registered) {
        success &= TheMdagMFermSystemSolverFactory::Instance().registerObject(std::string("GB300_CLOVER_INVERTER"),
                                                                               createFerm);
        registered = true;
      }
      return success;
    }
  }
}  // namespace Chroma
