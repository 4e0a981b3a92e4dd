// Krylov solvers on the device fields, batched over right-hand sides.
//
//   GBC_SOLVER_CG           LinOpSysSolverCG + InvCG2   (syssolver_linop_cg.h:57-96, invcg2.cc:70-232), FP64
//   GBC_SOLVER_RELIABLE_CG  LinOpSysSolverReliableCGClover + RelInvCG_a
//                           (syssolver_linop_rel_cg_clover.h:104-152, reliable_cg.cc:10-188):
//                           FP64 reliable updates around a CG whose vectors are FP32 and whose
//                           operator runs in the sloppy precision
//   GBC_SOLVER_MIXED        FP64 defect correction (the RICHARDSON_MP_CLOVER_INVERTER pattern,
//                           inv_multiprec_richardson.cc:13-107): each outer step recomputes the
//                           FP64 residual and solves for the correction with a CGNE whose operator
//                           and search vectors are in the sloppy precision and whose residual is
//                           refreshed from an FP32 operator (reliable updates)
//   GBC_SOLVER_FGMRES       FGMRES-DR(NKrylov, NDefl) (fgmres below; NDefl = 0 is plain restarted
//                           FGMRES), optionally preconditioned by the learned network (precond.cu),
//                           inside the same FP64 defect correction
//   GBC_SOLVER_BICGSTAB     the same FP64 defect correction around a reliable BiCGStab on M~
//                           (bicgstab.cu; RELIABLE_BICGSTAB_MP_CLOVER_INVERTER, reliable_bicgstab.cc:
//                           18-277); MdagM systems, and the rest of a solve whose inner BiCGStab broke
//                           down or raised the residual, use the inner CGNE
//
// Every right-hand side carries its own scalars on the device (CGScalars); a converged right-hand
// side keeps alpha = beta = 0 so that the batch can run on until the last one converges.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include <complex>

#include "ctx.h"
#include "dense.h"
#include "krylov.h"

namespace gbc {

namespace {

enum {
  SLOT_X = 1, SLOT_B, SLOT_R, SLOT_P, SLOT_MP, SLOT_MMP, SLOT_TE, SLOT_T1, SLOT_T2, SLOT_TEH,
  SLOT_XD, SLOT_BD, SLOT_RD, SLOT_TD1, SLOT_TD2, SLOT_TED, SLOT_ES, SLOT_RS, SLOT_CHIE, SLOT_PSIE, SLOT_SE,
  SLOT_XS, SLOT_RHS, SLOT_CHIO
};

struct Batch {
  int nrhs;
  std::vector<double> v;
};

// result[0][r] -> host (synchronises)
std::vector<double> fetch(gbc_ctx* c, int nred, int nrhs) {
  GBC_CUDA(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(double) * nred * nrhs, cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  return std::vector<double>(c->h_result, c->h_result + nred * nrhs);
}

std::vector<double> norm2(gbc_ctx* c, const Spinor& x) {
  blas_norm2(c->g, x, red(c), c->stream);
  return fetch(c, 1, x.nrhs);
}

// out = A x with A = M~ (normal = false) or M~^dag M~ (normal = true); |out|^2 not needed
void apply_sys(gbc_ctx* c, int prec, bool normal, const Spinor& x, const Spinor& out, const Spinor& t, const Spinor& te) {
  if (normal) {
    apply_meo(c, prec, false, x, t, te, false);
    apply_meo(c, prec, true, t, out, te, false);
  } else {
    apply_meo(c, prec, false, x, out, te, false);
  }
}

struct CgCfg {
  int pa, po;        // accumulator / operator precision
  double rsd;        // relative target on the normal-equation residual
  int maxit;
  double delta;      // reliable-update trigger (0: none)
  int check_every;   // host convergence checks
  const double* shift = nullptr;  // device, per right-hand side: solve (M~^dag M~ + shift) x = b
};

struct CgStats {
  std::vector<int> iters;
  std::vector<int> status;
  int reliable = 0;
};

// CG on M~^dag M~ x = b (InvCG2 recursion) with per-right-hand-side device scalars.
// active[r] == 0 skips right-hand side r (its x is left unchanged).
CgStats cg_normal(gbc_ctx* c, const CgCfg& cfg, const Spinor& x, const Spinor& b, bool zero_x,
                  const std::vector<int>& active) {
  const int n = x.nrhs;
  const Geom& g = c->g;
  cudaStream_t s = c->stream;
  Spinor r = sub(workspace(c, SLOT_R + 100 * pidx(cfg.pa), cfg.pa, n), 0, n);
  Spinor p = sub(workspace(c, SLOT_P + 100 * pidx(cfg.po), cfg.po, n), 0, n);
  Spinor mp = sub(workspace(c, SLOT_MP + 100 * pidx(cfg.po), cfg.po, n), 0, n);
  Spinor mmp = sub(workspace(c, SLOT_MMP + 100 * pidx(cfg.po), cfg.po, n), 0, n);
  Spinor te = sub(workspace(c, SLOT_TE + 100 * pidx(cfg.po), cfg.po, n), 0, n);
  CgStats st;
  st.iters.assign(n, 0);
  st.status.assign(n, GBC_OK);

  auto true_residual = [&]() {
    // r = b - A^dag A x in the accumulator precision
    Spinor t1 = sub(workspace(c, SLOT_T1 + 100 * pidx(cfg.pa), cfg.pa, n), 0, n);
    Spinor teh = sub(workspace(c, SLOT_TEH + 100 * pidx(cfg.pa), cfg.pa, n), 0, n);
    apply_sys(c, cfg.pa, true, x, r, t1, teh);
    if (cfg.shift) blas_shift_axpy(g, cfg.shift, x, r, s);
    blas_xmy_norm2(g, b, r, red(c), s);
  };
  if (zero_x) {
    blas_zero(g, x, s);
    blas_copy(g, r, b, s);
    blas_norm2(g, r, red(c), s);
  } else {
    true_residual();
  }
  std::vector<double> rr = fetch(c, 1, n);
  std::vector<double> bb = norm2(c, b);
  std::vector<CGScalars> hs(n);
  std::vector<double> maxrr(n), last_rel(n, HUGE_VAL), at_update(n);
  std::vector<int> stall(n, 0);
  for (int i = 0; i < n; ++i) {
    CGScalars& q = hs[i];
    std::memset(&q, 0, sizeof(q));
    q.c = q.cp = rr[i];
    q.c_prev = rr[i];
    q.rsd_sq = cfg.rsd * cfg.rsd * bb[i];
    q.active = active[i] && std::isfinite(rr[i]) && rr[i] > q.rsd_sq;
    if (!std::isfinite(rr[i]) || !std::isfinite(bb[i])) st.status[i] = GBC_ERR_NONFINITE;
    maxrr[i] = at_update[i] = std::sqrt(rr[i]);
  }
  GBC_CUDA(cudaMemcpyAsync(c->d_cg, hs.data(), sizeof(CGScalars) * n, cudaMemcpyHostToDevice, s));
  blas_copy(g, p, r, s);
  bool any = false;
  for (int i = 0; i < n; ++i) any |= hs[i].active != 0;
  // One iteration, all scalars on the device: no host round trip inside.
  auto body = [&]() {
    if (cfg.shift) {
      // mmp = (M~^dag M~ + shift) p and p^dag mmp -> result
      apply_meo(c, cfg.po, false, p, mp, te, false);
      apply_meo(c, cfg.po, true, mp, mmp, te, false);
      blas_shift_dot(g, cfg.shift, p, mmp, red(c), s);
      cg_alpha(c->d_cg, c->d_result, c->d_a, n, s);
    } else {
      apply_meo(c, cfg.po, false, p, mp, te, true);     // |mp|^2 -> result
      cg_alpha(c->d_cg, c->d_result, c->d_a, n, s);
      apply_meo(c, cfg.po, true, mp, mmp, te, false);
    }
    blas_cg_update(g, c->d_a, x, p, r, mmp, red(c), s);  // |r|^2 -> result
    cg_beta(c->d_cg, c->d_result, c->d_b, n, s);
    blas_xpay(g, r, c->d_b, p, s);                     // p = r + b p (b = 0 once converged)
  };
  // Blocks of kBlock iterations between host checks, replayed from a CUDA graph captured after
  // the first (uncaptured) iteration has run the autotuner on every kernel shape it needs.
  // A right-hand side that converges inside a block is frozen by alpha = beta = 0.
  constexpr int kBlock = 4;
  cudaGraphExec_t exec = nullptr;
  long long graph_launches = 0;
  int k = 0;
  while (any && k < cfg.maxit) {
    const int steps = k == 0 ? 1 : std::min(kBlock, cfg.maxit - k);
    if (k > 0 && steps == kBlock && c->use_graphs) {
      if (!exec) {
        cudaGraph_t graph;
        const long long l0 = launch_count();
        GBC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int q = 0; q < kBlock; ++q) body();
        GBC_CUDA(cudaStreamEndCapture(s, &graph));
        GBC_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        cudaGraphDestroy(graph);
        graph_launches = launch_count() - l0;
        count_launch(-graph_launches);
      }
      GBC_CUDA(cudaGraphLaunch(exec, s));
      count_launch(graph_launches);
    } else {
      for (int q = 0; q < steps; ++q) body();
    }
    k += steps;
    {
      GBC_CUDA(cudaMemcpyAsync(c->h_cg, c->d_cg, sizeof(CGScalars) * n, cudaMemcpyDeviceToHost, s));
      sync(c);
      any = false;
      bool trigger = false;
      for (int i = 0; i < n; ++i) {
        if (!std::isfinite(c->h_cg[i].cp)) st.status[i] = GBC_ERR_NONFINITE;
        if (!c->h_cg[i].active) continue;
        any = true;
        double rn = std::sqrt(c->h_cg[i].cp);
        maxrr[i] = std::max(maxrr[i], rn);
        if (cfg.delta > 0 && rn < cfg.delta * maxrr[i]) trigger = true;
        // an iterated residual back above its value at the last reliable update means the
        // recurrence has lost touch with the true residual (the accumulator precision's floor):
        // check it now, so that the stall test below can end this right-hand side instead of
        // letting the recurrence drift
        if (rn > at_update[i]) trigger = true;
      }
      if (any && trigger) {
        // reliable update: r = b - A^dag A x from the accumulator-precision operator
        true_residual();
        std::vector<double> nr = fetch(c, 1, n);
        std::memcpy(hs.data(), c->h_cg, sizeof(CGScalars) * n);
        std::vector<double> bnew(n);
        for (int i = 0; i < n; ++i) {
          CGScalars& q = hs[i];
          if (q.active) {
            q.b = q.c_prev > 0 ? nr[i] / q.c_prev : 0.0;
            q.c = q.cp = nr[i];
            maxrr[i] = at_update[i] = std::sqrt(nr[i]);
            // the true residual has hit the accumulator precision's floor when three reliable
            // updates in a row fail to halve it: stop this right-hand side (the outer FP64 loop
            // takes over from there)
            stall[i] = nr[i] > 0.25 * last_rel[i] ? stall[i] + 1 : 0;
            last_rel[i] = nr[i];
            if (!(nr[i] > q.rsd_sq) || stall[i] >= 3) {
              q.active = 0;
              q.b = 0;
            }
          }
          bnew[i] = q.b;
        }
        GBC_CUDA(cudaMemcpyAsync(c->d_cg, hs.data(), sizeof(CGScalars) * n, cudaMemcpyHostToDevice, s));
        sync(c);
        ++st.reliable;
      }
      if (!any) break;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  GBC_CUDA(cudaMemcpyAsync(c->h_cg, c->d_cg, sizeof(CGScalars) * n, cudaMemcpyDeviceToHost, s));
  sync(c);
  for (int i = 0; i < n; ++i) {
    st.iters[i] = c->h_cg[i].iters;
    if (c->h_cg[i].active && st.status[i] == GBC_OK) st.status[i] = GBC_ERR_NOT_CONVERGED;
  }
  return st;
}

// Chroma's RelInvCG_a, batched: b, psi in FP64; x, r in FP32; p, mp, mmp in the sloppy precision.
CgStats reliable_cg(gbc_ctx* c, int po, const Spinor& psi, const Spinor& chi, double rsd, double delta, int maxit) {
  const int n = psi.nrhs;
  const Geom& g = c->g;
  cudaStream_t s = c->stream;
  const int D = PREC_DOUBLE, S = PREC_SINGLE;
  Spinor b = sub(workspace(c, SLOT_BD, D, n), 0, n);
  Spinor rd = sub(workspace(c, SLOT_RD, D, n), 0, n);
  Spinor xd = sub(workspace(c, SLOT_XD, D, n), 0, n);
  Spinor t1 = sub(workspace(c, SLOT_TD1, D, n), 0, n);
  Spinor ted = sub(workspace(c, SLOT_TED, D, n), 0, n);
  Spinor x = sub(workspace(c, SLOT_XS, S, n), 0, n);
  Spinor r = sub(workspace(c, SLOT_RS, S, n), 0, n);
  Spinor p = sub(workspace(c, SLOT_P + 100 * pidx(po), po, n), 0, n);
  Spinor mp = sub(workspace(c, SLOT_MP + 100 * pidx(po), po, n), 0, n);
  Spinor mmp = sub(workspace(c, SLOT_MMP + 100 * pidx(po), po, n), 0, n);
  Spinor te = sub(workspace(c, SLOT_TE + 100 * pidx(po), po, n), 0, n);
  CgStats st;
  st.iters.assign(n, 0);
  st.status.assign(n, GBC_OK);
  std::vector<double> chi_norm = norm2(c, chi);
  // b = chi - A psi
  apply_sys(c, D, true, psi, b, t1, ted);
  blas_xmy_norm2(g, chi, b, red(c), s);
  std::vector<double> r_sq = fetch(c, 1, n);
  blas_copy(g, r, b, s);
  blas_zero(g, x, s);
  std::vector<double> rNorm(n), r0Norm(n), maxrx(n), maxrr(n), cc(n, 0.0), rsd_sq(n);
  std::vector<int> conv(n, 0);
  for (int i = 0; i < n; ++i) {
    rsd_sq[i] = rsd * rsd * chi_norm[i];
    rNorm[i] = r0Norm[i] = maxrx[i] = maxrr[i] = std::sqrt(r_sq[i]);
    if (r_sq[i] < rsd_sq[i]) conv[i] = 1;
  }
  std::vector<double> hb(n), ha(n);
  int k;
  auto all_conv = [&]() {
    for (int i = 0; i < n; ++i)
      if (!conv[i]) return false;
    return true;
  };
  for (k = 0; k < maxit && !all_conv(); ++k) {
    if (k == 0) {
      blas_copy(g, p, r, s);
    } else {
      for (int i = 0; i < n; ++i) hb[i] = conv[i] ? 0.0 : r_sq[i] / cc[i];
      GBC_CUDA(cudaMemcpyAsync(c->d_b, hb.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
      blas_xpay(g, r, c->d_b, p, s);
    }
    cc = r_sq;
    apply_meo(c, po, false, p, mp, te, true);
    std::vector<double> d = fetch(c, 1, n);
    apply_meo(c, po, true, mp, mmp, te, false);
    for (int i = 0; i < n; ++i) ha[i] = (conv[i] || !(d[i] > 0)) ? 0.0 : cc[i] / d[i];
    GBC_CUDA(cudaMemcpyAsync(c->d_a, ha.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    blas_cg_update(g, c->d_a, x, p, r, mmp, red(c), s);
    std::vector<double> nr = fetch(c, 1, n);
    bool updR = false, updX = false;
    for (int i = 0; i < n; ++i) {
      if (conv[i]) continue;
      ++st.iters[i];
      r_sq[i] = nr[i];
      if (!std::isfinite(nr[i])) {
        st.status[i] = GBC_ERR_NONFINITE;
        conv[i] = 1;
        continue;
      }
      rNorm[i] = std::sqrt(r_sq[i]);
      maxrx[i] = std::max(maxrx[i], rNorm[i]);
      maxrr[i] = std::max(maxrr[i], rNorm[i]);
      bool ux = rNorm[i] < delta * r0Norm[i] && r0Norm[i] <= maxrx[i];
      bool ur = (rNorm[i] < delta * maxrr[i] && r0Norm[i] <= maxrr[i]) || ux;
      updX |= ux;
      updR |= ur;
    }
    if (updR) {
      // r_dble = b - A (x promoted); r = r_dble (reliable_cg.cc:120-139)
      blas_copy(g, xd, x, s);
      apply_sys(c, D, true, xd, rd, t1, ted);
      blas_xmy_norm2(g, b, rd, red(c), s);
      std::vector<double> rr = fetch(c, 1, n);
      blas_copy(g, r, rd, s);
      ++st.reliable;
      for (int i = 0; i < n; ++i) {
        if (conv[i]) continue;
        r_sq[i] = rr[i];
        rNorm[i] = std::sqrt(rr[i]);
        maxrr[i] = rNorm[i];
      }
      if (updX) {
        // group-wise x update (reliable_cg.cc:141-151), for the whole batch
        blas_xpy(g, psi, xd, s);
        blas_zero(g, x, s);
        blas_copy(g, b, rd, s);
        for (int i = 0; i < n; ++i) {
          if (conv[i]) continue;
          r0Norm[i] = rNorm[i];
          maxrx[i] = rNorm[i];
        }
      }
    }
    for (int i = 0; i < n; ++i)
      if (!conv[i] && r_sq[i] < rsd_sq[i]) conv[i] = 1;
  }
  blas_xpy(g, psi, x, s);
  for (int i = 0; i < n; ++i)
    if (!conv[i] && st.status[i] == GBC_OK) st.status[i] = GBC_ERR_NOT_CONVERGED;
  return st;
}

// Batched right-preconditioned FGMRES-DR(m, k) on M~ x = b (FlexibleArnoldiT + Givens +
// LeastSquaresSolve, syssolver_linop_fgmres_dr.{h:31-148, cc:77-195, 256-273, 459-765}).  Krylov
// vectors in precision pa, operator in po; the preconditioner (learned network) maps V_j to Z_j,
// or Z_j = V_j.  One classical Gram-Schmidt pass per Arnoldi step.  Stops a right-hand side when
// |g_{j+1}| <= tol |b|.
// Deflated restarts (k = ndefl > 0, Morgan's GMRES-DR in the flexible form of the reference,
// :520-700): after a cycle of dimension d, the k harmonic Ritz vectors of smallest modulus -- here
// the Schur vectors of H_d + f h^H, f = H_d^-H h, h^H the last row of H, which span the same
// invariant subspace as the reference's eigenvectors -- and the cycle's least-squares residual
// c - H eta form G_{k+1}; with its orthonormal factor Q_{k+1} the next cycle starts from
// V' = V Q_{k+1}, Z' = Z Q_k, H' = Q_{k+1}^H H Q_k and c' = V'^H r, and its Arnoldi process extends
// the basis from column k.  Each right-hand side keeps its own H, Q and rotations.
CgStats fgmres(gbc_ctx* c, int pa, int po, const Spinor& x, const Spinor& b, double tol, int maxit, int m, int kdef,
               bool use_precond, const std::vector<int>& active0) {
  using cd = std::complex<double>;
  const int n = x.nrhs;
  const Geom& g = c->g;
  cudaStream_t s = c->stream;
  if (m < 1) m = 1;
  if (m > kMaxKrylov - 1) m = kMaxKrylov - 1;
  kdef = std::max(0, std::min(kdef, kMaxKrylov - 1 - m));
  const int mk = m + kdef;  // columns of a deflated cycle
  const int ldh = mk + 1;
  VecList V, Z, NV, NZ;
  for (int j = 0; j <= mk; ++j) V.v[j] = sub(workspace(c, 300 + j, pa, n), 0, n);
  const bool prec = use_precond && c->precond != nullptr;
  for (int j = 0; j < mk; ++j) Z.v[j] = prec ? sub(workspace(c, 340 + j, pa, n), 0, n) : V.v[j];
  Spinor w = sub(workspace(c, 380, pa, n), 0, n);
  Spinor oin = sub(workspace(c, 381, po, n), 0, n);
  Spinor oout = sub(workspace(c, 382, po, n), 0, n);
  Spinor te = sub(workspace(c, 383, po, n), 0, n);
  if (kdef > 0) {
    for (int t = 0; t <= kdef; ++t) NV.v[t] = sub(workspace(c, 400 + t, pa, n), 0, n);
    if (prec)
      for (int t = 0; t < kdef; ++t) NZ.v[t] = sub(workspace(c, 440 + t, pa, n), 0, n);
  }
  Red kred{c->d_kpartials, c->kpart_stride, c->d_kresult};
  CgStats st;
  st.iters.assign(n, 0);
  st.status.assign(n, GBC_OK);
  std::vector<double> bb = norm2(c, b);
  std::vector<int> done(n);
  for (int i = 0; i < n; ++i) done[i] = !active0[i];
  auto apply_A = [&](const Spinor& in, const Spinor& out) {
    if (po == pa) {
      apply_meo(c, po, false, in, out, te, false);
    } else {
      blas_copy(g, oin, in, s);
      apply_meo(c, po, false, oin, oout, te, false);
      blas_copy(g, out, oout, s);
    }
  };
  auto put_coef = [&](const std::vector<cd>& cf, int rows) {  // cf[row * n + rhs]
    // the staging buffer is pinned, so the copy reads it when the stream reaches it: wait for the
    // previous copy from it before overwriting (the deflated restart and the final x += Z eta
    // upload coefficients back to back)
    sync(c);
    for (size_t k = 0; k < cf.size(); ++k) c->h_kcoef[k] = make_double2(cf[k].real(), cf[k].imag());
    GBC_CUDA(cudaMemcpyAsync(c->d_kcoef, c->h_kcoef, sizeof(double2) * rows * n, cudaMemcpyHostToDevice, s));
  };
  auto fetch_dots = [&](int rows) {  // the rows of a multi_cdot, [row * n + rhs]
    GBC_CUDA(cudaMemcpyAsync(c->h_kresult, c->d_kresult, sizeof(double) * 2 * rows * n, cudaMemcpyDeviceToHost, s));
    sync(c);
    std::vector<cd> out((size_t)rows * n);
    for (int q = 0; q < rows; ++q)
      for (int i = 0; i < n; ++i)
        out[q * n + i] = cd(c->h_kresult[(q * 2 + 0) * n + i], c->h_kresult[(q * 2 + 1) * n + i]);
    return out;
  };
  int total = 0;
  Spinor tea = sub(workspace(c, 384, pa, n), 0, n);
  std::vector<double> prev_beta(n, HUGE_VAL);
  // kept from one cycle to the next for the deflated restart: the unrotated H (column-major,
  // ldh rows), the right-hand side c of the cycle's least-squares problem, its solution eta and
  // the cycle's dimension
  std::vector<std::vector<cd>> H(n, std::vector<cd>((size_t)ldh * mk, 0.0)), cvec(n, std::vector<cd>(ldh, 0.0));
  std::vector<std::vector<cd>> eta_prev(n);
  std::vector<int> prev_dim(n, 0);
  int cycle = 0;
  while (total < maxit) {
    // r = b - A x with the operator in the vectors' precision: each restart is a refinement step,
    // so the cycles may run on the cheaper sloppy operator
    apply_meo(c, pa, false, x, w, tea, false);
    blas_xmy_norm2(g, b, w, red(c), s);
    std::vector<double> rr = fetch(c, 1, n);
    std::vector<double> beta(n);
    bool all = true;
    for (int i = 0; i < n; ++i) {
      beta[i] = std::sqrt(rr[i]);
      if (!std::isfinite(beta[i])) {
        st.status[i] = GBC_ERR_NONFINITE;
        done[i] = 1;
      }
      if (!done[i] && beta[i] <= tol * std::sqrt(bb[i])) done[i] = 1;
      // a cycle that no longer reduces the true residual has reached the precision floor
      if (!done[i] && beta[i] > 0.9 * prev_beta[i]) done[i] = 1;
      prev_beta[i] = beta[i];
      all &= done[i] != 0;
    }
    if (all) break;
    // a deflated restart needs a previous cycle longer than the deflation space on every
    // right-hand side still running
    bool deflate = kdef > 0 && cycle > 0;
    for (int i = 0; i < n && deflate; ++i)
      if (!done[i] && prev_dim[i] <= kdef) deflate = false;
    const int kc = deflate ? kdef : 0;
    // per right-hand side: R (column-major, R[col][row]), g, the Givens rotations of the cycle's
    // columns (c, s), and for a deflated cycle the rotations (row pairs) that triangularised H'
    std::vector<std::vector<cd>> R(n, std::vector<cd>((size_t)ldh * mk, 0.0)), gv(n, std::vector<cd>(ldh, 0.0));
    std::vector<std::vector<cd>> gc(n, std::vector<cd>(mk)), gs(n, std::vector<cd>(mk));
    std::vector<std::vector<int>> qrow(n);
    std::vector<std::vector<cd>> qc(n), qs(n);
    std::vector<int> dim(n, kc), cyc_done(done);
    // rotation (A, B) -> (conj(c) A + conj(s) B, -s A + c B) on rows (r, r + 1) of a vector
    auto rot = [](std::vector<cd>& v, int r, cd cc, cd ss, size_t off) {
      const cd A = v[off + r], B = v[off + r + 1];
      v[off + r] = std::conj(cc) * A + std::conj(ss) * B;
      v[off + r + 1] = -ss * A + cc * B;
    };
    auto givens = [](cd f, cd gg, cd& cc, cd& ss) -> cd {  // syssolver_linop_fgmres_dr.h:31-148
      if (f == 0.0) {
        cc = 0.0;
        ss = 1.0;
        return gg;
      }
      if (gg == 0.0) {
        ss = 0.0;
        cc = f / std::abs(f);  // rot() maps f to conj(cc) f = |f|
        return std::abs(f);
      }
      const double t = std::sqrt(std::norm(f) + std::norm(gg));
      cc = f / t;
      ss = gg / t;
      return t;
    };
    if (!deflate) {
      std::vector<cd> a(n);
      for (int i = 0; i < n; ++i) a[i] = done[i] ? 0.0 : 1.0 / beta[i];
      put_coef(a, 1);
      blas_cax(g, c->d_kcoef, w, V.v[0], s);
      for (int i = 0; i < n; ++i) {
        std::fill(H[i].begin(), H[i].end(), cd(0.0));
        std::fill(cvec[i].begin(), cvec[i].end(), cd(0.0));
        gv[i][0] = cvec[i][0] = beta[i];
      }
    } else {
      // Q_{k+1} per right-hand side (column-major, (d + 1) x (k + 1)) and H' = Q_{k+1}^H H Q_k
      std::vector<std::vector<cd>> Qk(n), Hn(n);
      int dmax = 0;
      for (int i = 0; i < n; ++i) {
        if (done[i]) continue;
        const int d = prev_dim[i];
        dmax = std::max(dmax, d);
        std::vector<cd> Hd((size_t)d * d), f(d);
        for (int col = 0; col < d; ++col) {
          for (int row = 0; row < d; ++row) Hd[(size_t)col * d + row] = H[i][(size_t)col * ldh + row];
          f[col] = std::conj(H[i][(size_t)col * ldh + d]);  // h = (last row of H)^H
        }
        std::vector<cd> Am = Hd, Y;
        if (!dense::lu_solve(d, Hd, f, true)) throw std::string("FGMRES-DR: singular Hessenberg block");
        for (int col = 0; col < d; ++col)
          for (int row = 0; row < d; ++row) Am[(size_t)col * d + row] += f[row] * H[i][(size_t)col * ldh + d];
        if (!dense::schur(d, Am, Y)) throw std::string("FGMRES-DR: harmonic Ritz values did not converge");
        dense::sort_smallest(d, Am, Y, kc);
        std::vector<cd> G((size_t)(d + 1) * (kc + 1), 0.0), Rg;
        for (int col = 0; col < kc; ++col)
          for (int row = 0; row < d; ++row) G[(size_t)col * (d + 1) + row] = Y[(size_t)col * d + row];
        for (int row = 0; row <= d; ++row) {
          cd v = cvec[i][row];
          for (int col = 0; col < d; ++col) v -= H[i][(size_t)col * ldh + row] * eta_prev[i][col];
          G[(size_t)kc * (d + 1) + row] = v;
        }
        dense::qr_thin(d + 1, kc + 1, G, Rg);
        // H Q_k ((d + 1) x k), then Q_{k+1}^H (H Q_k)
        std::vector<cd> HQ((size_t)(d + 1) * kc, 0.0);
        for (int col = 0; col < kc; ++col)
          for (int row = 0; row <= d; ++row) {
            cd v = 0.0;
            for (int q = 0; q < d; ++q) v += H[i][(size_t)q * ldh + row] * G[(size_t)col * (d + 1) + q];
            HQ[(size_t)col * (d + 1) + row] = v;
          }
        Hn[i].assign((size_t)(kc + 1) * kc, 0.0);
        for (int col = 0; col < kc; ++col)
          for (int row = 0; row <= kc; ++row) {
            cd v = 0.0;
            for (int q = 0; q <= d; ++q) v += std::conj(G[(size_t)row * (d + 1) + q]) * HQ[(size_t)col * (d + 1) + q];
            Hn[i][(size_t)col * (kc + 1) + row] = v;
          }
        Qk[i] = G;
      }
      // the new basis: V'_t = sum_j V_j Q(j, t), Z'_t = sum_j Z_j Q(j, t) (per right-hand side)
      for (int t = 0; t <= kc; ++t) {
        std::vector<cd> cf((size_t)(dmax + 1) * n, 0.0);
        for (int i = 0; i < n; ++i)
          if (!done[i])
            for (int j = 0; j <= prev_dim[i]; ++j) cf[(size_t)j * n + i] = Qk[i][(size_t)t * (prev_dim[i] + 1) + j];
        put_coef(cf, dmax + 1);
        blas_zero(g, NV.v[t], s);
        multi_caxpy(g, V, dmax + 1, c->d_kcoef, NV.v[t], 1.0, s);
        if (prec && t < kc) {
          blas_zero(g, NZ.v[t], s);
          multi_caxpy(g, Z, dmax, c->d_kcoef, NZ.v[t], 1.0, s);
        }
      }
      for (int t = 0; t <= kc; ++t) blas_copy(g, V.v[t], NV.v[t], s);
      if (prec)
        for (int t = 0; t < kc; ++t) blas_copy(g, Z.v[t], NZ.v[t], s);
      // c' = V'^H r
      multi_cdot(g, V, kc + 1, w, kred, s);
      std::vector<cd> cn = fetch_dots(kc + 1);
      for (int i = 0; i < n; ++i) {
        std::fill(H[i].begin(), H[i].end(), cd(0.0));
        std::fill(cvec[i].begin(), cvec[i].end(), cd(0.0));
        if (done[i]) continue;
        for (int col = 0; col < kc; ++col)
          for (int row = 0; row <= kc; ++row) H[i][(size_t)col * ldh + row] = Hn[i][(size_t)col * (kc + 1) + row];
        for (int row = 0; row <= kc; ++row) cvec[i][row] = gv[i][row] = cn[(size_t)row * n + i];
        // triangularise H' (full, (k + 1) x k) by rotations of adjacent rows, bottom up per column;
        // the same rotations go to g now and to the first k + 1 rows of every later column
        std::vector<cd> Hw = Hn[i];
        for (int col = 0; col < kc; ++col)
          for (int row = kc; row > col; --row) {
            cd cc, ss;
            const cd rv = givens(Hw[(size_t)col * (kc + 1) + row - 1], Hw[(size_t)col * (kc + 1) + row], cc, ss);
            for (int c2 = col; c2 < kc; ++c2) rot(Hw, row - 1, cc, ss, (size_t)c2 * (kc + 1));
            Hw[(size_t)col * (kc + 1) + row - 1] = rv;
            Hw[(size_t)col * (kc + 1) + row] = 0.0;
            rot(gv[i], row - 1, cc, ss, 0);
            qrow[i].push_back(row - 1);
            qc[i].push_back(cc);
            qs[i].push_back(ss);
          }
        for (int col = 0; col < kc; ++col)
          for (int row = 0; row <= kc; ++row) R[i][(size_t)col * ldh + row] = Hw[(size_t)col * (kc + 1) + row];
      }
    }
    int j;
    for (j = kc; j < mk && j - kc < m && total < maxit; ++j) {
      if (prec) precond_apply(c, V.v[j], Z.v[j]);
      apply_A(Z.v[j], w);
      std::vector<cd> h((j + 1) * n, 0.0);
      // one Gram-Schmidt pass, as the reference's FlexibleArnoldi (syssolver_linop_fgmres_dr.cc:
      // 108-111, modified Gram-Schmidt); here the classical form, so that all j + 1 products come
      // from one batched multi-dot.  A second pass took 30 % of the time and changed no iteration
      // count on the propagator and the 16^3x32 workloads (the FP64 outer residual checks anyway).
      {
        multi_cdot(g, V, j + 1, w, kred, s);
        std::vector<cd> dots = fetch_dots(j + 1);
        std::vector<cd> hp((j + 1) * n);
        for (int q = 0; q <= j; ++q)
          for (int i = 0; i < n; ++i) {
            cd v = dots[q * n + i];
            if (cyc_done[i]) v = 0.0;
            hp[q * n + i] = -v;
            h[q * n + i] += v;
          }
        put_coef(hp, j + 1);
        multi_caxpy(g, V, j + 1, c->d_kcoef, w, 1.0, s);
      }
      std::vector<double> wn2 = norm2(c, w);
      ++total;
      std::vector<cd> inv(n, 0.0);
      for (int i = 0; i < n; ++i) {
        if (cyc_done[i]) continue;
        ++st.iters[i];
        const double wn = std::sqrt(wn2[i]);
        std::vector<cd>& Ri = R[i];
        const size_t col = (size_t)j * ldh;
        for (int q = 0; q <= j; ++q) H[i][col + q] = Ri[col + q] = h[q * n + i];
        H[i][col + j + 1] = Ri[col + j + 1] = wn;
        // the deflated restart's rotations (rows 0 .. k), then the cycle's own
        for (size_t t = 0; t < qrow[i].size(); ++t) rot(Ri, qrow[i][t], qc[i][t], qs[i][t], col);
        for (int q = kc; q < j; ++q) rot(Ri, q, gc[i][q], gs[i][q], col);
        const cd rv = givens(Ri[col + j], Ri[col + j + 1], gc[i][j], gs[i][j]);
        Ri[col + j] = rv;
        Ri[col + j + 1] = 0.0;
        rot(gv[i], j, gc[i][j], gs[i][j], 0);
        dim[i] = j + 1;
        const double est = std::abs(gv[i][j + 1]);
        if (!std::isfinite(est)) {
          st.status[i] = GBC_ERR_NONFINITE;
          cyc_done[i] = done[i] = 1;
          continue;
        }
        // converged, or exact (happy) breakdown of the Arnoldi process
        if (est <= tol * std::sqrt(bb[i]) || wn < 1e-14 * std::sqrt(bb[i])) cyc_done[i] = 1;
        else inv[i] = 1.0 / wn;
      }
      put_coef(inv, 1);
      blas_cax(g, c->d_kcoef, w, V.v[j + 1], s);
      bool everyone = true;
      for (int i = 0; i < n; ++i) everyone &= cyc_done[i] != 0;
      if (everyone) {
        ++j;
        break;
      }
    }
    // least squares R eta = g per right-hand side, then x += Z eta
    const int jmax = std::min(j, mk);
    std::vector<cd> eta((size_t)jmax * n, 0.0);
    for (int i = 0; i < n; ++i) {
      const int d = dim[i];
      prev_dim[i] = d;
      if (d == 0 || done[i]) continue;
      std::vector<cd> e(d);
      for (int row = d - 1; row >= 0; --row) {
        cd v = gv[i][row];
        for (int col = row + 1; col < d; ++col) v -= R[i][(size_t)col * ldh + row] * e[col];
        e[row] = v / R[i][(size_t)row * ldh + row];
      }
      for (int q = 0; q < d; ++q) eta[q * n + i] = e[q];
      eta_prev[i] = e;
    }
    if (jmax > 0) {
      put_coef(eta, jmax);
      multi_caxpy(g, Z, jmax, c->d_kcoef, x, 1.0, s);
    }
    ++cycle;
  }
  for (int i = 0; i < n; ++i)
    if (!done[i] && st.status[i] == GBC_OK) st.status[i] = GBC_ERR_NOT_CONVERGED;
  return st;
}

}  // namespace

std::vector<int> refine_shifted(gbc_ctx* c, int sloppy, const Spinor& chi, const double* d_shift,
                                const Spinor& psi, const std::vector<double>& rsd, int max_iter,
                                std::vector<double>& rr, std::vector<int>& status) {
  const int D = PREC_DOUBLE, S = PREC_SINGLE;
  const int n = psi.nrhs;
  const Geom& g = c->g;
  cudaStream_t s = c->stream;
  Spinor r = sub(workspace(c, 760, D, n), 0, n);
  Spinor t1 = sub(workspace(c, 761, D, n), 0, n);
  Spinor te = sub(workspace(c, 762, D, n), 0, n);
  Spinor rs = sub(workspace(c, 763, S, n), 0, n);
  Spinor es = sub(workspace(c, 764, S, n), 0, n);
  Spinor chib = chi;  // every right-hand-side index reads the one source
  chib.nrhs = n;
  chib.rhs_bytes = 0;
  chib.norm_rhs_stride = 0;
  const double chi2 = norm2(c, chi)[0];
  std::vector<int> iters(n, 0), done(n, 0);
  status.assign(n, GBC_OK);
  rr.assign(n, 0.0);
  std::vector<double> prev(n, HUGE_VAL);
  for (int outer = 0; outer < 30; ++outer) {
    // FP64 residual of every shifted system
    apply_sys(c, D, true, psi, r, t1, te);
    blas_shift_axpy(g, d_shift, psi, r, s);
    blas_xmy_norm2(g, chib, r, red(c), s);
    rr = fetch(c, 1, n);
    std::vector<int> active(n, 0);
    bool any = false;
    double worst = 0.0;
    int budget = max_iter;
    for (int q = 0; q < n; ++q) {
      if (done[q]) continue;
      if (!std::isfinite(rr[q])) {
        status[q] = GBC_ERR_NONFINITE;
        done[q] = 1;
        continue;
      }
      // converged, or a correction that no longer halves the residual (the sloppy floor)
      if (rr[q] <= rsd[q] * rsd[q] * chi2 || rr[q] > 0.25 * prev[q]) {
        done[q] = 1;
        continue;
      }
      prev[q] = rr[q];
      active[q] = 1;
      any = true;
      worst = std::max(worst, std::sqrt(rr[q] / chi2) / rsd[q]);
      budget = std::min(budget, max_iter - iters[q]);
    }
    if (!any || budget <= 0) break;
    // the correction only needs the part of the reduction still missing (with a factor 2 margin)
    const double itol = std::min(0.1, std::max(1e-6, 0.5 / worst));
    blas_copy(g, rs, r, s);
    CgCfg cfg{S, sloppy, itol, budget, 0.1, 1, d_shift};
    CgStats st = cg_normal(c, cfg, es, rs, true, active);
    for (int q = 0; q < n; ++q) {
      if (!active[q]) continue;
      iters[q] += st.iters[q];
      if (st.status[q] == GBC_ERR_NONFINITE) {
        status[q] = GBC_ERR_NONFINITE;
        done[q] = 1;
      }
    }
    blas_xpy(g, psi, es, s);
  }
  for (int q = 0; q < n; ++q)
    if (status[q] == GBC_OK && !(rr[q] <= rsd[q] * rsd[q] * chi2)) status[q] = GBC_ERR_NOT_CONVERGED;
  return iters;
}

int solve_device(gbc_ctx* c, const gbc_solve_params* pp, int nrhs, double* psi_canon, const double* chi_canon,
                 gbc_result* res, const std::function<void()>* after_export) {
  gbc_solve_params p = *pp;
  if (!(p.rsd_target > 0)) p.rsd_target = 1e-10;
  if (p.max_iter <= 0) p.max_iter = 10000;
  if (!(p.delta > 0)) p.delta = 0.1;
  if (!(p.rsd_tolerance_factor > 0)) p.rsd_tolerance_factor = 10.0;
  if (!(p.inner_tol > 0)) p.inner_tol = 1e-6;
  if (p.inner_max_iter <= 0) p.inner_max_iter = p.max_iter;
  if (p.nkrylov <= 0) p.nkrylov = 16;
  if (p.ndefl < 0 || p.ndefl + std::min(p.nkrylov, kMaxKrylov - 1) > kMaxKrylov - 1) {
    c->err = "NDefl + NKrylov above 32";
    return GBC_ERR_ARGS;
  }
  int sloppy = p.sloppy_precision ? p.sloppy_precision : c->opts.sloppy_precision;
  if (sloppy != PREC_HALF && sloppy != PREC_SINGLE && sloppy != PREC_DOUBLE) return GBC_ERR_ARGS;
  if (p.system < GBC_SYS_MEO || p.system > GBC_SYS_SYM_MDAGM) return GBC_ERR_ARGS;
  if (p.solver < GBC_SOLVER_CG || p.solver > GBC_SOLVER_BICGSTAB) return GBC_ERR_ARGS;
  // the symmetric operator M_s: every solver below runs unchanged, apply_meo applies M_s
  const bool symmetric = p.system == GBC_SYS_SYM || p.system == GBC_SYS_SYM_MDAGM;
  if (symmetric) {
    if (p.use_precond) {
      c->err = "the learned preconditioner approximates M~^-1, not the symmetric operator's inverse";
      return GBC_ERR_ARGS;
    }
    p.system = p.system == GBC_SYS_SYM ? GBC_SYS_MEO : GBC_SYS_MDAGM;
  }
  SymScope sym_scope(c, symmetric);

  const int D = PREC_DOUBLE;
  const Geom& g = c->g;
  cudaStream_t s = c->stream;
  const size_t rs = (size_t)c->V * 24;
  ensure_prec(c, D);
  if (p.solver != GBC_SOLVER_CG) {
    ensure_prec(c, sloppy);
    ensure_prec(c, PREC_SINGLE);
  }
  // For the full system, the Schur prep and the intermediate residuals of the defect correction
  // run in double-float arithmetic on the FP64 fields (about 1e-14 relative, far below any
  // target): GB300 executes FP32 at a large multiple of its FP64 rate.  The solution's
  // reconstruction and the final true residual stay FP64.  The odd-site systems keep FP64
  // residuals, whose last one is also their final check; GBC_OUTER_DF=0 (and the symmetric
  // operator) keeps every step in FP64.
  const char* odf = getenv("GBC_OUTER_DF");
  const int DX = (odf && odf[0] == '0') || symmetric || p.system != GBC_SYS_FULL ? D : PREC_DF;
  if (DX == PREC_DF) ensure_prec(c, PREC_DF);
  // In the defect correction the Schur-prepared source chi'_o only seeds the first inner solve,
  // whose tolerance is far coarser than FP32 rounding, so it is formed with the FP32 operator;
  // every outer residual then comes from the original source instead of chi'_o,
  //   r = chi_o - A_oo psi + 1/2 D_oe A_ee^-1 (chi_e + 1/2 D_eo psi)   (= chi'_o - M~ psi),
  // in double-float arithmetic: one stencil launch fewer in that arithmetic per solve.
  const bool approx_prep = DX == PREC_DF && !c->act.twisted && sloppy != PREC_DOUBLE &&
                           (p.solver == GBC_SOLVER_MIXED || p.solver == GBC_SOLVER_FGMRES ||
                            p.solver == GBC_SOLVER_BICGSTAB);
  if (symmetric) {
    // A_oo^-1 packed before any iteration is captured into a graph
    ensure_sym(c, D);
    if (p.solver != GBC_SOLVER_CG) {
      ensure_sym(c, sloppy);
      ensure_sym(c, PREC_SINGLE);
    }
  }
  cudaEvent_t ev0, ev1;
  GBC_CUDA(cudaEventCreate(&ev0));
  GBC_CUDA(cudaEventCreate(&ev1));
  GBC_CUDA(cudaEventRecord(ev0, s));
  const long long launches0 = launch_count();
  const int n = nrhs;
  Spinor chi = sub(workspace(c, SLOT_B, D, n), 0, n);    // odd right-hand side of the odd system
  Spinor psi = sub(workspace(c, SLOT_X, D, n), 0, n);    // odd solution
  Spinor t1 = sub(workspace(c, SLOT_TD1, D, n), 0, n);
  Spinor t2 = sub(workspace(c, SLOT_TD2, D, n), 0, n);
  Spinor ted = sub(workspace(c, SLOT_TED, D, n), 0, n);
  const PrecFields& fd = c->pf[pidx(D)];

  import_spinor(g, chi_canon, rs, 1, chi, s);
  Spinor chie, psie, chio;
  std::vector<double> src_no, src_ne, src_np;  // |chi_o|^2, |chi_e|^2, |chi'_o|^2 of the full system
  if (p.system == GBC_SYS_FULL) {
    // Schur prep (eoprec_fermact_qprop.cc:47-54): chi'_o = chi_o - (-1/2 D_oe) A_ee^-1 chi_e
    chie = sub(workspace(c, SLOT_CHIE, D, n), 0, n);
    psie = sub(workspace(c, SLOT_PSIE, D, n), 0, n);
    import_spinor(g, chi_canon, rs, 0, chie, s);
    src_no = norm2(c, chi);
    src_ne = norm2(c, chie);
    if (approx_prep) {
      chio = sub(workspace(c, SLOT_CHIO, D, n), 0, n);
      blas_copy(g, chio, chi, s);
      // the FP32 fields of the inner solver's workspaces (the same slots and precision below)
      Spinor ae = sub(workspace(c, SLOT_ES, PREC_SINGLE, n), 0, n);
      Spinor at = sub(workspace(c, SLOT_RS, PREC_SINGLE, n), 0, n);
      blas_copy(g, ae, chie, s);
      apply_clover(c, PREC_SINGLE, 0, true, ae, at);
      hop(c, PREC_SINGLE, 1, HOP_PLAIN, false, 0.5, at, ae, nullptr, nullptr, false);
      blas_xpy(g, chi, ae, s);
    } else {
      apply_clover(c, DX, 0, true, chie, ted);
      hop(c, DX, 1, HOP_PLAIN, false, 0.5, ted, t1, nullptr, nullptr, false);
      blas_xpy(g, chi, t1, s);
    }
    // the even reconstruction is exact, so the full residual equals the odd one: solve the odd
    // system to target * |chi| / |chi'_o| so that |M psi - chi| / |chi| meets the target
    src_np = norm2(c, chi);
    double scale = 1.0;
    for (int i = 0; i < n; ++i)
      if (src_np[i] > 0) scale = std::min(scale, std::sqrt((src_no[i] + src_ne[i]) / src_np[i]));
    p.rsd_target *= scale;
  }
  if (p.zero_guess) blas_zero(g, psi, s);
  else import_spinor(g, psi_canon, rs, 1, psi, s);

  const bool mdagm = p.system == GBC_SYS_MDAGM;
  std::vector<int> iters(n, 0), status(n, GBC_OK), outer(n, 0);
  int reliable = 0;
  // |chi - A psi|^2 in FP64 for the final psi, when the solver has just computed it (the last
  // outer residual of the defect correction, the last restart check of CG): the final check
  // then reuses it instead of applying the FP64 operator again
  std::vector<double> known_rr;

  if (p.solver == GBC_SOLVER_CG) {
    // chi' = M~^dag chi (LinOp) ; InvCG2 on M~^dag M~
    Spinor rhs = chi;
    if (!mdagm) {
      rhs = sub(workspace(c, SLOT_RHS, D, n), 0, n);
      apply_meo(c, D, true, chi, rhs, ted, false);
    }
    // CGNE stops on |M^dag r| <= RsdCG |M^dag chi|; the true residual of M psi = chi can end
    // slightly above the target, so restart from the current psi with a tightened tolerance until
    // the FP64 true residual meets it (Chroma's optional restart, syssolver_linop_cg.h:73-81)
    std::vector<int> active(n, 1);
    std::vector<double> bb = norm2(c, chi);
    double tol = p.rsd_target;
    for (int pass = 0; pass < 4; ++pass) {
      int budget = p.max_iter;
      for (int i = 0; i < n; ++i) budget = std::min(budget, p.max_iter - iters[i]);
      if (budget <= 0) break;
      CgCfg cfg{D, D, tol, budget, 0.0, 4};
      CgStats st = cg_normal(c, cfg, psi, rhs, pass == 0 && p.zero_guess != 0, active);
      for (int i = 0; i < n; ++i) {
        if (!active[i]) continue;
        iters[i] += st.iters[i];
        status[i] = st.status[i];
      }
      apply_sys(c, D, mdagm, psi, t1, t2, ted);
      blas_xmy_norm2(g, chi, t1, red(c), s);
      std::vector<double> rr = fetch(c, 1, n);
      known_rr = rr;
      double worst_rel = 0;
      bool any = false;
      for (int i = 0; i < n; ++i) {
        double relr = bb[i] > 0 ? std::sqrt(rr[i] / bb[i]) : 0.0;
        active[i] = status[i] == GBC_OK && relr > p.rsd_target;
        if (active[i]) {
          any = true;
          worst_rel = std::max(worst_rel, relr);
        }
      }
      if (!any) break;
      tol *= 0.5 * p.rsd_target / worst_rel;
    }
  } else if (p.solver == GBC_SOLVER_RELIABLE_CG) {
    Spinor rhs = chi;
    if (!mdagm) {
      rhs = sub(workspace(c, SLOT_RHS, D, n), 0, n);
      apply_meo(c, D, true, chi, rhs, ted, false);
    }
    int po = sloppy == PREC_DOUBLE ? PREC_SINGLE : sloppy;
    CgStats st = reliable_cg(c, po, psi, rhs, p.rsd_target, p.delta, p.max_iter);
    iters = st.iters;
    status = st.status;
    reliable = st.reliable;
  } else if (p.solver == GBC_SOLVER_MIXED || p.solver == GBC_SOLVER_FGMRES || p.solver == GBC_SOLVER_BICGSTAB) {
    // FP64 defect correction: r = chi - A psi; solve A e = r in low precision; psi += e
    const int S = PREC_SINGLE;
    const int pa = sloppy == PREC_DOUBLE ? D : S;
    Spinor rd = sub(workspace(c, SLOT_RD, D, n), 0, n);
    Spinor rsl = sub(workspace(c, SLOT_RS, pa, n), 0, n);
    Spinor es = sub(workspace(c, SLOT_ES, pa, n), 0, n);
    Spinor rhs = sub(workspace(c, SLOT_SE, pa, n), 0, n);
    Spinor teh = sub(workspace(c, SLOT_TEH + 50, pa, n), 0, n);
    std::vector<double> bb = src_np.size() == (size_t)n ? src_np : norm2(c, chi);
    std::vector<int> done(n, 0);
    for (int i = 0; i < n; ++i)
      if (!std::isfinite(bb[i])) {
        status[i] = GBC_ERR_NONFINITE;
        done[i] = 1;
      }
    const int max_outer = 50;
    int total = 0;
    std::vector<double> prev_rr(n, HUGE_VAL);
    bool rr_exact = false;  // whether the last residual came from the FP64 operator
    // BiCGStab can break down (rho or (r0, v) -> 0) or stagnate where CG on the normal equations
    // cannot: once an inner BiCGStab breaks down or its correction is taken back, the remaining
    // outer steps of this solve run the inner CGNE instead
    bool bicg_fallback = false;
    for (int it = 0; it <= max_outer; ++it) {
      bool rr_is_bb = false;
      if (it == 0 && p.zero_guess) {
        blas_copy(g, rd, chi, s);  // r = chi, |r|^2 = bb
        rr_is_bb = true;
        rr_exact = true;
      } else if (it >= 2 && pa != D && p.system == GBC_SYS_FULL) {
        // From the third outer step on, r <- r - A e with A applied to the last correction e in
        // the accumulator precision: its error, ~1e-7 |r| of the step before, is far below the
        // target once that residual is small, and the full system ends with its FP64 residual
        // over both parities as the check.  Saves one FP64 operator per step (FP64 is slow here).
        Spinor ta = sub(workspace(c, SLOT_XS + 50, pa, n), 0, n);
        Spinor tb = sub(workspace(c, SLOT_XS + 51, pa, n), 0, n);
        apply_sys(c, pa, mdagm, es, ta, tb, teh);
        blas_xsub_norm2(g, rd, ta, red(c), s);
        rr_exact = false;
      } else if (approx_prep) {
        // r = chi_o - (A_oo psi - 1/2 D_oe A_ee^-1 (chi_e + 1/2 D_eo psi)) from the original
        // source, in double-float arithmetic on the FP64 fields
        hop(c, DX, 0, HOP_PLAIN, false, 0.5, psi, ted, nullptr, nullptr, false);
        blas_xpy(g, ted, chie, s);
        apply_clover(c, DX, 0, true, ted, t2);
        hop(c, DX, 1, HOP_XPAY, false, -0.5, t2, rd, &psi, c->pf[pidx(DX)].clov[1], false);
        blas_xmy_norm2(g, chio, rd, red(c), s);
        rr_exact = false;
      } else {
        // residual with the FP64 fields (double-float arithmetic unless GBC_OUTER_DF=0)
        apply_sys(c, DX, mdagm, psi, rd, t2, ted);
        blas_xmy_norm2(g, chi, rd, red(c), s);
        rr_exact = DX == D;
      }
      std::vector<double> rr = rr_is_bb ? bb : fetch(c, 1, n);
      // A correction that left the FP64 residual larger than before (an inner solve that broke
      // down) is taken back, and that right-hand side stops with the better iterate.
      bool revert = false;
      const bool retry_cg = p.solver == GBC_SOLVER_BICGSTAB && !bicg_fallback;
      for (int i = 0; i < n; ++i) {
        const bool back = !done[i] && std::isfinite(prev_rr[i]) && !(rr[i] <= prev_rr[i]);
        c->h_coef[i] = make_double2(back ? -1.0 : 0.0, 0.0);
        c->h_coef[n + i] = make_double2(1.0, 0.0);
        if (back) {
          revert = true;
          rr[i] = prev_rr[i];
          if (retry_cg) {
            bicg_fallback = true;  // this right-hand side goes on with the inner CGNE
          } else {
            done[i] = 1;
            if (status[i] == GBC_OK) status[i] = GBC_ERR_NOT_CONVERGED;
          }
        }
      }
      if (revert) {
        GBC_CUDA(cudaMemcpyAsync(c->d_ca, c->h_coef, sizeof(double2) * n, cudaMemcpyHostToDevice, s));
        GBC_CUDA(cudaMemcpyAsync(c->d_cb, c->h_coef + n, sizeof(double2) * n, cudaMemcpyHostToDevice, s));
        blas_axpby(g, c->d_ca, es, c->d_cb, psi, s);  // psi = psi - es for those right-hand sides
        sync(c);
      }
      for (int i = 0; i < n; ++i) prev_rr[i] = rr[i];
      bool all = true;
      double worst = 0.0;
      for (int i = 0; i < n; ++i) {
        if (done[i]) continue;
        if (!std::isfinite(rr[i])) {
          status[i] = GBC_ERR_NONFINITE;
          done[i] = 1;
          continue;
        }
        if (rr[i] <= p.rsd_target * p.rsd_target * bb[i]) done[i] = 1;
        else {
          all = false;
          worst = std::max(worst, std::sqrt(rr[i] / bb[i]));
        }
      }
      if (all || it == max_outer || total >= p.max_iter) {
        if (rr_exact) known_rr = rr;
        break;
      }
      std::vector<int> active(n);
      for (int i = 0; i < n; ++i) {
        active[i] = !done[i];
        if (active[i]) ++outer[i];
      }
      // inner right-hand side in the accumulator precision
      blas_copy(g, rsl, rd, s);
      // never ask the inner solve for more than the outer target needs: the reduction still
      // missing is target / worst, taken with a factor 2 of margin (but no looser than 0.1)
      double need = 0.5 * p.rsd_target / worst;
      double itol = std::min(0.1, std::max(p.inner_tol, need));
      CgStats st;
      if (p.solver == GBC_SOLVER_FGMRES && !mdagm) {
        // flexible GMRES on M~ e = r directly (preconditioned by the learned network if loaded)
        blas_zero(g, es, s);
        st = fgmres(c, pa, sloppy, es, rsl, itol, p.inner_max_iter, p.nkrylov, p.ndefl, p.use_precond != 0, active);
      } else if (p.solver == GBC_SOLVER_BICGSTAB && !mdagm && !bicg_fallback) {
        // BiCGStab on M~ e = r directly (no normal equations)
        InnerStats bs = bicgstab(c, pa, sloppy, itol, p.inner_max_iter, p.delta, es, rsl, active);
        st.iters = bs.iters;
        st.status = bs.status;
        st.reliable = bs.reliable;
        for (int i = 0; i < n; ++i)
          if (active[i] && st.status[i] == GBC_ERR_BREAKDOWN) {
            bicg_fallback = true;
            st.status[i] = GBC_OK;  // the correction so far is kept; CGNE takes over
          }
      } else {
        if (!mdagm) apply_meo(c, pa, true, rsl, rhs, teh, false);
        else blas_copy(g, rhs, rsl, s);
        CgCfg cfg{pa, sloppy, itol, p.inner_max_iter, p.delta, 1};
        st = cg_normal(c, cfg, es, rhs, true, active);
      }
      reliable += st.reliable;
      int mx = 0;
      for (int i = 0; i < n; ++i) {
        iters[i] += st.iters[i];
        mx = std::max(mx, st.iters[i]);
        if (st.status[i] == GBC_ERR_NONFINITE) {
          status[i] = GBC_ERR_NONFINITE;
          done[i] = 1;
        }
      }
      total += mx;
      blas_xpy(g, psi, es, s);
    }
    for (int i = 0; i < n; ++i)
      if (!done[i] && status[i] == GBC_OK) status[i] = GBC_ERR_NOT_CONVERGED;
  }

  // true FP64 residual of the system solved, then even reconstruction for the full system
  // (the full system reports the residual of M over both parities, computed below instead)
  std::vector<double> bb = p.system == GBC_SYS_FULL ? std::vector<double>(n, 0.0) : norm2(c, chi);
  std::vector<double> rr(n, 0.0);
  if (p.system != GBC_SYS_FULL) {
    if (known_rr.size() == (size_t)n) {
      rr = known_rr;
    } else {
      apply_sys(c, D, mdagm, psi, t1, t2, ted);
      blas_xmy_norm2(g, chi, t1, red(c), s);
      rr = fetch(c, 1, n);
    }
  }
  export_spinor(g, psi_canon, rs, 1, psi, s);
  if (p.system != GBC_SYS_FULL && after_export) (*after_export)();
  if (p.system == GBC_SYS_FULL) {
    // psi_e = A_ee^-1 (chi_e + 1/2 D_eo psi_o)   (eoprec_fermact_qprop.cc:60-67)
    hop(c, D, 0, HOP_PLAIN, false, 0.5, psi, t1, nullptr, nullptr, false);
    blas_xpy(g, t1, chie, s);
    apply_clover(c, D, 0, true, t1, psie);
    export_spinor(g, psi_canon, rs, 0, psie, s);
    if (after_export) (*after_export)();
    // full residual |M psi - chi| over both parities (eoprec_fermact_qprop.cc:70-76); the even
    // part A_ee psi_e - 1/2 D_eo psi_o - chi_e reuses t1 = chi_e + 1/2 D_eo psi_o from above
    Spinor ue = sub(workspace(c, SLOT_T2 + 50, D, n), 0, n);
    Spinor uo = sub(workspace(c, SLOT_T2, D, n), 0, n);
    apply_clover(c, D, 0, false, psie, ue);
    hop(c, D, 1, HOP_XPAY, false, -0.5, psie, uo, &psi, fd.clov[1], false);
    // the original odd source: kept from the Schur prep, else imported again
    Spinor src_o = chio;
    if (!approx_prep) {
      src_o = sub(workspace(c, SLOT_PSIE + 50, D, n), 0, n);
      import_spinor(g, chi_canon, rs, 1, src_o, s);
    }
    blas_xmy_norm2(g, t1, ue, red(c), s);
    std::vector<double> re = fetch(c, 1, n);
    blas_xmy_norm2(g, src_o, uo, red(c), s);
    std::vector<double> ro = fetch(c, 1, n);
    for (int i = 0; i < n; ++i) {
      rr[i] = re[i] + ro[i];
      bb[i] = src_ne[i] + src_no[i];
    }
  }
  GBC_CUDA(cudaGetLastError());
  GBC_CUDA(cudaEventRecord(ev1, s));
  GBC_CUDA(cudaEventSynchronize(ev1));
  float ms = 0;
  GBC_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  int worst = GBC_OK;
  for (int i = 0; i < n; ++i) {
    gbc_result& o = res[i];
    std::memset(&o, 0, sizeof(o));
    o.device_seconds = ms * 1e-3;
    o.launches = launch_count() - launches0;
    o.n_count = iters[i];
    o.resid = std::sqrt(rr[i]);
    o.rel_resid = bb[i] > 0 ? std::sqrt(rr[i] / bb[i]) : o.resid;
    o.n_outer = outer[i];
    o.n_reliable = reliable;
    o.status = status[i];
    if (!std::isfinite(o.resid)) o.status = GBC_ERR_NONFINITE;
    // RsdToleranceFactor check (syssolver_linop_clover_quda_w.h:636-643)
    if (o.status == GBC_ERR_NOT_CONVERGED && o.rel_resid <= p.rsd_tolerance_factor * p.rsd_target) o.status = GBC_OK;
    if (o.status == GBC_OK && !(o.rel_resid <= p.rsd_tolerance_factor * p.rsd_target)) o.status = GBC_ERR_NOT_CONVERGED;
    if (o.status != GBC_OK && worst == GBC_OK) worst = o.status;
  }
  return worst;
}

}  // namespace gbc
