// Multi-shift CG on the normal equations, (M~^dag M~ + sigma_s) psi_s = chi for every shift at
// once: the RHMC solver behind Chroma's MdagMMultiSysSolverCG (multi_syssolver_mdagm_cg.h:58-80)
// -> MInvCG2 (minvcg2.cc:70-357), Jegerlehner's recursion (hep-lat/9708029).  With a sloppy
// precision (HALF or SINGLE) the recursion runs in FP32 and each shift is then refined by an FP64
// defect correction whose corrections come from CG on the shifted system in the sloppy operator,
// Chroma's multiprec pattern (a single-precision MInvCG2 followed by per-shift refinement).  One Krylov space of
// the unshifted M~^dag M~ is built; each shifted solution follows from the ratios zeta_s of its
// residual to the unshifted one, so an iteration costs one M~^dag M~ plus one fused update of all
// shifted search vectors and one of all solutions.  Fields and sums in FP64, the scalar recursion
// on the host (two reductions per iteration).  The recursion, its sign conventions and its
// convergence test (|r| zeta_s <= RsdCG_s |chi|) are the reference's, so iteration counts agree.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "ctx.h"

namespace gbc {
namespace {

enum { MS_CHI = 700, MS_R, MS_P0, MS_MP, MS_MMP, MS_TE, MS_P, MS_X, MS_T1, MS_T2 };

// the first finalized sum of red(c) -> host (synchronises)
double fetch(gbc_ctx* c) {
  GBC_CUDA(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  sync(c);
  return c->h_result[0];
}
double norm2(gbc_ctx* c, const Spinor& x) {
  blas_norm2(c->g, x, red(c), c->stream);
  return fetch(c);
}

// every right-hand-side index of the view reads the same field x
Spinor broadcast(const Spinor& x, int n) {
  Spinor t = x;
  t.nrhs = n;
  t.rhs_bytes = 0;
  t.norm_rhs_stride = 0;
  return t;
}

struct Coefs {
  std::vector<double2> h;  // [2][n]
  double2* d = nullptr;
  int n = 0;
  explicit Coefs(int n_) : h(2 * (size_t)n_), n(n_) { GBC_CUDA(cudaMalloc(&d, sizeof(double2) * 2 * n_)); }
  ~Coefs() {
    if (d) cudaFree(d);
  }
  // upload a[s], b[s] and run y_s = a_s x_s + b_s y_s (then wait, the host vector is reused)
  void axpby(gbc_ctx* c, const Spinor& x, const Spinor& y) {
    GBC_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(double2) * 2 * n, cudaMemcpyHostToDevice, c->stream));
    blas_axpby(c->g, d, x, d + n, y, c->stream);
    sync(c);
  }
};

}  // namespace

int solve_multishift(gbc_ctx* c, const gbc_solve_params* pp, int ns, const double* shifts, const double* rsd,
                     double* const* psi_canon, const double* chi_canon, gbc_result* res) {
  const int D = PREC_DOUBLE;
  const Geom& g = c->g;
  cudaStream_t s = c->stream;
  const int max_iter = pp->max_iter > 0 ? pp->max_iter : 10000;
  // mixed precision (sloppy_precision HALF or SINGLE): the shared-Krylov recursion runs on FP32
  // fields and the FP32 operator to a relative 1e-6 (near FP32's floor), then every shift is
  // refined by the FP64 defect correction of refine_shifted (batched over the shifts, corrections
  // from CG in the sloppy operator); else the recursion runs in FP64 to the targets
  const int sp = pp->sloppy_precision;
  const bool mixed = sp == PREC_HALF || sp == PREC_SINGLE;
  const int W = mixed ? PREC_SINGLE : D;
  ensure_prec(c, D);
  if (mixed) {
    ensure_prec(c, PREC_SINGLE);
    ensure_prec(c, sp);
  }
  const double t0 = now();
  cudaEvent_t ev0, ev1;
  GBC_CUDA(cudaEventCreate(&ev0));
  GBC_CUDA(cudaEventCreate(&ev1));
  GBC_CUDA(cudaEventRecord(ev0, s));
  const long long launches0 = launch_count();

  const int o = 20 * pidx(W);  // workspace slots per recursion precision
  Spinor chid = sub(workspace(c, MS_CHI, D, 1), 0, 1);
  Spinor chi = mixed ? sub(workspace(c, MS_CHI + o, W, 1), 0, 1) : chid;
  Spinor r = sub(workspace(c, MS_R + o, W, 1), 0, 1);
  Spinor p0 = sub(workspace(c, MS_P0 + o, W, 1), 0, 1);
  Spinor mp = sub(workspace(c, MS_MP + o, W, 1), 0, 1);
  Spinor mmp = sub(workspace(c, MS_MMP + o, W, 1), 0, 1);
  Spinor te = sub(workspace(c, MS_TE + o, W, 1), 0, 1);
  Spinor P = sub(workspace(c, MS_P + o, W, ns), 0, ns);
  Spinor X = sub(workspace(c, MS_X + o, W, ns), 0, ns);
  const size_t rs = (size_t)c->V * 24;
  ensure_stage(c, ns);
  GBC_CUDA(cudaMemcpyAsync(c->d_stage[0], chi_canon, rs * sizeof(double), cudaMemcpyHostToDevice, s));
  import_spinor(g, c->d_stage[0], rs, 1, chid, s);
  if (mixed) blas_copy(g, chi, chid, s);
  Coefs co(ns), one(1);

  std::vector<double> shift(shifts, shifts + ns), rsd_sq(ns);
  std::vector<int> conv(ns, 0);
  int k = 0, iters = 0, status = GBC_OK;
  const double chi2 = norm2(c, chi);
  blas_zero(g, X, s);
  if (!(chi2 > 0.0)) {
    status = std::isfinite(chi2) ? GBC_OK : GBC_ERR_NONFINITE;
  } else {
    for (int q = 0; q < ns; ++q) {
      const double t = mixed ? std::max(rsd[q], 1e-6) : rsd[q];
      rsd_sq[q] = chi2 * t * t;
    }
    const int smallest = (int)(std::min_element(shift.begin(), shift.end()) - shift.begin());
    // r = p0 = p_s = chi
    blas_copy(g, r, chi, s);
    blas_copy(g, p0, chi, s);
    blas_copy(g, P, broadcast(chi, ns), s);
    // b = -|r|^2 / <p0, A p0>,  r += b A p0
    double cp = chi2;
    apply_meo(c, W, false, p0, mp, te, true);
    double d = fetch(c);
    apply_meo(c, W, true, mp, mmp, te, false);
    double b = -cp / d;
    one.h[0] = make_double2(b, 0.0);
    one.h[1] = make_double2(1.0, 0.0);
    one.axpby(c, mmp, r);
    // zeta_prev = 1, zeta = 1 / (1 - sigma b), bs = b zeta; psi_s = -bs chi
    std::vector<double> zprev(ns, 1.0), z(ns), bs(ns);
    for (int q = 0; q < ns; ++q) {
      z[q] = 1.0 / (1.0 - shift[q] * b);
      bs[q] = b * z[q];
      co.h[q] = make_double2(-bs[q], 0.0);
      co.h[ns + q] = make_double2(0.0, 0.0);
    }
    co.axpby(c, broadcast(chi, ns), X);
    double cc = norm2(c, r);
    bool done = cc < rsd_sq[smallest];
    for (k = 1; k <= max_iter && !done; ++k) {
      if (!std::isfinite(cc)) {
        status = GBC_ERR_NONFINITE;
        break;
      }
      const double a = cc / cp;
      // p0 = r + a p0
      one.h[0] = make_double2(1.0, 0.0);
      one.h[1] = make_double2(a, 0.0);
      one.axpby(c, r, p0);
      // p_s = zeta_s r + as_s p_s  (converged shifts keep p_s: coefficients 0, 1)
      for (int q = 0; q < ns; ++q) {
        if (conv[q]) {
          co.h[q] = make_double2(0.0, 0.0);
          co.h[ns + q] = make_double2(1.0, 0.0);
        } else {
          const double as = a * z[q] * bs[q] / (zprev[q] * b);
          co.h[q] = make_double2(z[q], 0.0);
          co.h[ns + q] = make_double2(as, 0.0);
        }
      }
      co.axpby(c, broadcast(r, ns), P);
      cp = cc;
      apply_meo(c, W, false, p0, mp, te, true);
      d = fetch(c);
      apply_meo(c, W, true, mp, mmp, te, false);
      const double bp = b;
      b = -cp / d;
      one.h[0] = make_double2(b, 0.0);
      one.h[1] = make_double2(1.0, 0.0);
      one.axpby(c, mmp, r);
      cc = norm2(c, r);
      // zeta_next = zeta zeta_prev bp / (b a (zeta_prev - zeta) + zeta_prev bp (1 - sigma b))
      for (int q = 0; q < ns; ++q) {
        if (conv[q]) continue;
        const double zn = z[q] * zprev[q] * bp / (b * a * (zprev[q] - z[q]) + zprev[q] * bp * (1.0 - shift[q] * b));
        bs[q] = b * zn / z[q];
        zprev[q] = z[q];
        z[q] = zn;
      }
      // psi_s -= bs_s p_s
      for (int q = 0; q < ns; ++q) {
        co.h[q] = make_double2(conv[q] ? 0.0 : -bs[q], 0.0);
        co.h[ns + q] = make_double2(1.0, 0.0);
      }
      co.axpby(c, P, X);
      done = true;
      for (int q = 0; q < ns; ++q) {
        if (!conv[q]) conv[q] = cc * z[q] * z[q] < rsd_sq[q];
        done = done && conv[q];
      }
      iters = k;
    }
    if (!done && status == GBC_OK) status = GBC_ERR_NOT_CONVERGED;
  }
  // mixed precision: FP64 copies of the solutions, refined shift by shift (batched)
  std::vector<int> refine_iters(ns, 0), refine_status(ns, GBC_OK);
  std::vector<double> refine_rr;
  Spinor XD = X;
  if (mixed) {
    XD = sub(workspace(c, MS_X, D, ns), 0, ns);
    blas_copy(g, XD, X, s);
    if (status == GBC_OK || status == GBC_ERR_NOT_CONVERGED) {
      double* d_shift = nullptr;
      GBC_CUDA(cudaMalloc(&d_shift, sizeof(double) * ns));
      GBC_CUDA(cudaMemcpyAsync(d_shift, shift.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, s));
      std::vector<double> rsdv(rsd, rsd + ns);
      try {
        refine_iters = refine_shifted(c, sp, chid, d_shift, XD, rsdv, std::max(1, max_iter - iters), refine_rr,
                                      refine_status);
      } catch (...) {
        cudaFree(d_shift);
        throw;
      }
      cudaFree(d_shift);
      status = GBC_OK;
    }
  }
  GBC_CUDA(cudaEventRecord(ev1, s));
  GBC_CUDA(cudaEventSynchronize(ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  const long long launches = launch_count() - launches0;

  // true FP64 residual of every shifted system, then the odd sites of each solution to the host
  // (the even sites of psi_s are kept: the caller's arrays are staged first)
  Spinor t1 = sub(workspace(c, MS_T1, D, 1), 0, 1);
  Spinor t2 = sub(workspace(c, MS_T2, D, 1), 0, 1);
  Spinor ted = sub(workspace(c, MS_TE, D, 1), 0, 1);
  for (int q = 0; q < ns; ++q) {
    Spinor xq = sub(XD, q, 1);
    apply_meo(c, D, false, xq, t1, ted, false);
    apply_meo(c, D, true, t1, t2, ted, false);
    one.h[0] = make_double2(shift[q], 0.0);
    one.h[1] = make_double2(1.0, 0.0);
    one.axpby(c, xq, t2);  // t2 = (M~^dag M~ + sigma) psi
    blas_xmy_norm2(g, chid, t2, red(c), s);
    const double rr = fetch(c);
    gbc_result& o = res[q];
    o = gbc_result{};
    o.n_count = iters + refine_iters[q];
    o.n_outer = mixed ? 1 : 0;
    o.resid = std::sqrt(rr);
    o.rel_resid = chi2 > 0 ? std::sqrt(rr / chi2) : 0.0;
    o.status = mixed && status == GBC_OK ? refine_status[q] : status;
    if (o.status == GBC_ERR_NOT_CONVERGED) o.status = GBC_OK;  // judged by the tolerance factor below
    if (o.status == GBC_OK && !(o.rel_resid <= pp->rsd_tolerance_factor * rsd[q])) o.status = GBC_ERR_NOT_CONVERGED;
    o.device_seconds = ms * 1e-3;
    o.launches = (int)launches;
    GBC_CUDA(cudaMemcpyAsync(c->d_stage[1], psi_canon[q], rs * sizeof(double), cudaMemcpyHostToDevice, s));
    export_spinor(g, c->d_stage[1], rs, 1, xq, s);
    GBC_CUDA(cudaMemcpyAsync(psi_canon[q], c->d_stage[1], rs * sizeof(double), cudaMemcpyDeviceToHost, s));
    sync(c);
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  const double t1s = now();
  int worst = GBC_OK;
  for (int q = 0; q < ns; ++q) {
    res[q].seconds = t1s - t0;
    if (res[q].status != GBC_OK && worst == GBC_OK) worst = res[q].status;
  }
  return worst;
}

}  // namespace gbc

using namespace gbc;

extern "C" int gbc_solve_multishift(gbc_ctx* c, const gbc_solve_params* p, int nshift, const double* shifts,
                                    const double* rsd_targets, double* const* psi, const double* chi,
                                    gbc_result* res) {
  if (!c || !p || nshift < 1 || !shifts || !psi || !chi || !res) return GBC_ERR_ARGS;
  for (int q = 0; q < nshift; ++q)
    if (!psi[q] || !std::isfinite(shifts[q]) || shifts[q] < 0.0) return GBC_ERR_ARGS;
  if (!c->have_gauge) {
    c->err = "load the gauge field first";
    return GBC_ERR_STATE;
  }
  std::vector<double> rsd(nshift);
  for (int q = 0; q < nshift; ++q) {
    rsd[q] = rsd_targets ? rsd_targets[q] : p->rsd_target;
    if (!(rsd[q] > 0)) rsd[q] = 1e-10;
  }
  gbc_solve_params pp = *p;
  if (!(pp.rsd_tolerance_factor > 0)) pp.rsd_tolerance_factor = 10.0;
  try {
    return solve_multishift(c, &pp, nshift, shifts, rsd.data(), psi, chi, res);
  } catch (const CudaError& e) {
    c->err = std::string(e.where) + ": " + cudaGetErrorString(e.e);
    return GBC_ERR_CUDA;
  } catch (const std::string& m) {
    c->err = m;
    return GBC_ERR_STATE;
  } catch (const std::bad_alloc&) {
    c->err = "host allocation failed";
    return GBC_ERR_CUDA;
  }
}
