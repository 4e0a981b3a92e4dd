/*! \file
 *  \brief quarkProp4GB300: the spin-colour sources of a propagator as one device batch.
 */
#include "chroma_plugin/quarkprop4_gb300_w.h"

#include <cmath>
#include <sstream>
#include <vector>

#include "chroma_plugin/syssolver_linop_clover_gb300_w.h"
#include "util/ferm/transf.h"

namespace Chroma
{
  void quarkProp4GB300(LatticePropagator& q_sol, XMLWriter& xml_out, const LatticePropagator& q_src,
                       Handle<FermState<LatticeFermion, multi1d<LatticeColorMatrix>, multi1d<LatticeColorMatrix> > > state,
                       const GroupXML_t& invParam, QuarkSpinType quarkSpinType, int& ncg_had)
  {
    START_CODE();
    push(xml_out, "QuarkProp4");
    ncg_had = 0;
    // the spin columns solved, as quarkProp4_a (quarkprop4_w.cc:47-64)
    int start_spin = 0, end_spin = Ns;
    if (quarkSpinType == QUARK_SPIN_TYPE_UPPER) end_spin = Ns / 2;
    if (quarkSpinType == QUARK_SPIN_TYPE_LOWER) start_spin = Ns / 2;
    const int nspin = end_spin - start_spin;
    const int n = Nc * nspin;

    std::istringstream is(invParam.xml);
    XMLReader paramtop(is);
    SysSolverGB300CloverParams p(paramtop, invParam.path);
    if (p.MaxRHS < n) p.MaxRHS = n;
    GB300CloverContext dev(state, p);

    // sources in quarkProp4_a's order (colour outer, spin inner), each scaled to unit norm
    const long V = Layout::vol();
    const size_t per = (size_t)V * 24;
    std::vector<double> chi((size_t)n * per), psi((size_t)n * per, 0.0), buf;
    std::vector<double> scale(n, 1.0);
    for (int color_source = 0; color_source < Nc; ++color_source)
      for (int spin_source = start_spin; spin_source < end_spin; ++spin_source) {
        const int k = color_source * nspin + (spin_source - start_spin);
        LatticeFermion f;
        PropToFerm(q_src, f, color_source, spin_source);
        dev.gather(buf, f);
        double nrm = 0;
        for (double v : buf) nrm += v * v;
        nrm = std::sqrt(nrm);
        const double fact = nrm != 0.0 ? 1.0 / nrm : 1.0;
        for (size_t i = 0; i < per; ++i) chi[k * per + i] = buf[i] * fact;
        scale[k] = 1.0 / fact;
      }

    gbc_solve_params q;
    q.solver = p.SolverType == "CG" ? GBC_SOLVER_CG
             : p.SolverType == "RELIABLE_CG" ? GBC_SOLVER_RELIABLE_CG
             : (p.SolverType == "FGMRES" || p.SolverType == "GCR") ? GBC_SOLVER_FGMRES
             : p.SolverType == "BICGSTAB" ? GBC_SOLVER_BICGSTAB : GBC_SOLVER_MIXED;
    q.system = GBC_SYS_FULL;
    q.rsd_target = toDouble(p.RsdTarget);
    q.max_iter = p.MaxIter;
    q.delta = toDouble(p.Delta);
    q.rsd_tolerance_factor = toDouble(p.RsdToleranceFactor);
    q.sloppy_precision = p.CudaSloppyPrecision == "DOUBLE" ? GBC_PREC_DOUBLE
                       : p.CudaSloppyPrecision == "SINGLE" ? GBC_PREC_SINGLE : GBC_PREC_HALF;
    q.inner_tol = toDouble(p.InnerTol);
    q.inner_max_iter = 0;
    q.nkrylov = p.NKrylov;
    q.ndefl = p.NDefl;
    q.use_precond = p.PrecondWeights.empty() ? 0 : 1;
    q.zero_guess = 1;  // quarkProp4_a starts every source from psi = zero
    std::vector<gbc_result> res(n);
    for (gbc_result& r : res) {
      r = gbc_result{};
      r.resid = std::nan("");
    }
    const int rc = gbc_solve(dev.get(), &q, n, psi.data(), chi.data(), res.data());
    if (rc != GBC_OK) {
      QDPIO::cerr << "GB300_CLOVER_INVERTER (batched propagator): " << gbc_strerror(rc) << ": "
                  << gbc_last_error(dev.get()) << std::endl;
      if (!p.SilentFail) QDP_abort(1);
    }

    for (int color_source = 0; color_source < Nc; ++color_source)
      for (int spin_source = start_spin; spin_source < end_spin; ++spin_source) {
        const int k = color_source * nspin + (spin_source - start_spin);
        ncg_had += res[k].n_count;
        push(xml_out, "Qprop");
        write(xml_out, "color_source", color_source);
        write(xml_out, "spin_source", spin_source);
        write(xml_out, "n_count", res[k].n_count);
        write(xml_out, "resid", Real(res[k].resid));
        pop(xml_out);
        buf.assign(psi.begin() + k * per, psi.begin() + (k + 1) * per);
        for (double& v : buf) v *= scale[k];
        LatticeFermion f;
        dev.scatter(f, buf, 3);  // both parities
        FermToProp(f, q_sol, color_source, spin_source);
        // UPPER / LOWER: the other half's columns are the negated copies (quarkprop4_w.cc:120-175)
        if (quarkSpinType != QUARK_SPIN_TYPE_FULL) {
          for (double& v : buf) v = -v;
          LatticeFermion g;
          dev.scatter(g, buf, 3);
          const int other = quarkSpinType == QUARK_SPIN_TYPE_UPPER ? spin_source + Ns / 2 : spin_source - Ns / 2;
          FermToProp(g, q_sol, color_source, other);
        }
      }
    pop(xml_out);
    END_CODE();
  }
}  // namespace Chroma
