// gbc_blas: the BLAS-1 kernels the solvers run, applied to host fields through the C ABI, so that
// their reductions and fused updates can be checked on their own against QDP++'s norm2 and
// innerProduct (FP64 "Double" sums) and the update formulas of InvCG2 and BiCGStab
// (lib/actions/ferm/invert/invcg2.cc:165-221, invbicgstab.cc:89-160).
//
// Every field is nrhs canonical full-lattice spinors back to back; the kernels see their odd
// checkerboard (rb[1], the subset of the even-odd solves).  A field is imported into the precision
// of its role (accumulator or operator precision, as the solvers store it), the kernel runs once,
// and the fields it updates are exported back over the odd sites (even sites keep the caller's
// values).
#include <cstring>
#include <string>

#include "ctx.h"

using namespace gbc;

namespace {

bool valid_prec(int p) { return p == GBC_PREC_DOUBLE || p == GBC_PREC_SINGLE || p == GBC_PREC_HALF; }

}  // namespace

extern "C" int gbc_blas(gbc_ctx* c, int op, int prec_acc, int prec_op, int nrhs, const double* coef,
                        double* const* fields, double* res) {
  if (!c || !fields || nrhs < 1 || nrhs > c->max_rhs || op < GBC_BLAS_NORM2 || op > GBC_BLAS_BICG_XR)
    return GBC_ERR_ARGS;
  if (!valid_prec(prec_acc) || !valid_prec(prec_op)) return GBC_ERR_ARGS;
  static const int nfields[] = {1, 2, 4, 2, 6};
  for (int k = 0; k < nfields[op]; ++k)
    if (!fields[k]) return GBC_ERR_ARGS;
  if ((op == GBC_BLAS_NORM2 || op == GBC_BLAS_CDOT || op == GBC_BLAS_CG_UPDATE || op == GBC_BLAS_BICG_XR) && !res)
    return GBC_ERR_ARGS;
  if ((op == GBC_BLAS_CG_UPDATE || op == GBC_BLAS_XPAY || op == GBC_BLAS_BICG_XR) && !coef) return GBC_ERR_ARGS;
  try {
    ensure_stage(c, nrhs);
    cudaStream_t st = c->stream;
    const size_t rs = (size_t)c->V * 24;
    const size_t bytes = (size_t)nrhs * rs * sizeof(double);
    auto import = [&](int k, int prec) {
      Spinor f = sub(workspace(c, 1100 + 4 * k + pidx(prec), prec, nrhs), 0, nrhs);
      GBC_CUDA(cudaMemcpyAsync(c->d_stage[0], fields[k], bytes, cudaMemcpyHostToDevice, st));
      import_spinor(c->g, c->d_stage[0], rs, 1, f, st);
      return f;
    };
    auto export_back = [&](int k, const Spinor& f) {
      GBC_CUDA(cudaMemcpyAsync(c->d_stage[1], fields[k], bytes, cudaMemcpyHostToDevice, st));
      export_spinor(c->g, c->d_stage[1], rs, 1, f, st);
      GBC_CUDA(cudaMemcpyAsync(fields[k], c->d_stage[1], bytes, cudaMemcpyDeviceToHost, st));
      sync(c);
    };
    auto results = [&](int nq) {
      // device rows [q][rhs] -> res[rhs * nq + q]
      GBC_CUDA(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(double) * nq * nrhs, cudaMemcpyDeviceToHost, st));
      sync(c);
      for (int r = 0; r < nrhs; ++r)
        for (int q = 0; q < nq; ++q) res[r * nq + q] = c->h_result[q * nrhs + r];
    };
    switch (op) {
      case GBC_BLAS_NORM2: {
        Spinor x = import(0, prec_op);
        blas_norm2(c->g, x, red(c), st);
        results(1);
        break;
      }
      case GBC_BLAS_CDOT: {
        Spinor x = import(0, prec_acc);
        Spinor y = import(1, prec_op);
        blas_cdot(c->g, x, y, red(c), st);
        results(2);
        break;
      }
      case GBC_BLAS_CG_UPDATE: {
        Spinor x = import(0, prec_acc), p = import(1, prec_op), r = import(2, prec_acc), q = import(3, prec_op);
        GBC_CUDA(cudaMemcpyAsync(c->d_a, coef, sizeof(double) * nrhs, cudaMemcpyHostToDevice, st));
        blas_cg_update(c->g, c->d_a, x, p, r, q, red(c), st);
        results(1);
        export_back(0, x);
        export_back(2, r);
        break;
      }
      case GBC_BLAS_XPAY: {
        Spinor r = import(0, prec_acc), p = import(1, prec_op);
        GBC_CUDA(cudaMemcpyAsync(c->d_b, coef, sizeof(double) * nrhs, cudaMemcpyHostToDevice, st));
        blas_xpay(c->g, r, c->d_b, p, st);
        export_back(1, p);
        break;
      }
      case GBC_BLAS_BICG_XR: {
        Spinor x = import(0, prec_acc), r = import(1, prec_acc), p = import(2, prec_op), v = import(3, prec_op),
               t = import(4, prec_op), r0 = import(5, prec_acc);
        bicgstab_xr_update(c, prec_acc, prec_op, coef, nrhs, x, r, p, v, t, r0);
        results(3);
        export_back(0, x);
        export_back(1, r);
        break;
      }
    }
    GBC_CUDA(cudaGetLastError());
    sync(c);
    return GBC_OK;
  } catch (const CudaError& e) {
    c->err = std::string(e.where) + ": " + cudaGetErrorString(e.e);
    return GBC_ERR_CUDA;
  } catch (const std::string& s) {
    c->err = s;
    return GBC_ERR_ARGS;
  }
}
