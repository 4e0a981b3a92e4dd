// Host-side context of the C ABI: device fields, workspaces and the operator building blocks
// shared by the solvers.
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/gbclover.h"
#include "gbc_kernels.h"

namespace gbc {

// index of a precision's device fields in gbc_ctx::pf (PREC_DF: the double-float split copies)
inline int pidx(int prec) {
  return prec == PREC_DOUBLE ? 0 : prec == PREC_SINGLE ? 1 : prec == PREC_HALF ? 2 : 3;
}

struct PrecFields {
  bool ready = false;
  int recon = 18;
  void* gauge[2][4] = {{nullptr}};  // [parity][mu]
  void* clov[2] = {nullptr, nullptr};
  void* clovinv = nullptr;      // A^-1, even parity
  void* clovinv_odd = nullptr;  // A^-1, odd parity (symmetric operator only; packed on first use)
};

struct CudaError {
  cudaError_t e;
  std::string where;
};

// throws CudaError on failure
void cuda_check(cudaError_t e, const char* where);
#define GBC_CUDA(x) ::gbc::cuda_check((x), #x)

}  // namespace gbc

struct gbc_ctx {
  int dims[4];
  long V = 0;
  gbc::Geom g{};
  gbc_action act{};
  gbc_opts opts{};
  cudaStream_t stream = nullptr;
  std::string err;
  bool have_gauge = false;
  long gauge_version = 0;  // bumped by every gbc_load_gauge
  double link_coeff[4] = {1, 1, 1, 1};

  // canonical FP64 copies on the device
  double* d_links = nullptr;  // [V][4][3][3] complex = 72 doubles per site
  double* d_clov = nullptr;   // [V][72]
  double* d_inv = nullptr;    // [V][72] A^-1 (both parities)
  double logdet_even = 0;  // sum over even sites of log|d| of A's LDL^dag factors
  double logdet_odd = 0;   // the same over the odd sites
  int nneg = 0;

  gbc::PrecFields pf[4];  // FP64, FP32, FP16 fields and the double-float copies of the FP64 ones

  // reductions and CG scalars
  int max_rhs = 12;
  int part_stride = 0;
  double* d_partials = nullptr;
  double* d_result = nullptr;
  double* h_result = nullptr;  // pinned
  gbc::CGScalars* d_cg = nullptr;
  gbc::CGScalars* h_cg = nullptr;  // pinned
  double* d_a = nullptr;
  double* d_b = nullptr;
  double2* d_ca = nullptr;
  double2* d_cb = nullptr;
  double2* h_coef = nullptr;  // pinned, 2 * max_rhs

  // block-vector reductions of the flexible GMRES: partials [2*33][max_rhs][blas blocks],
  // results [2*33][max_rhs], coefficients [33][max_rhs] (device + pinned host mirrors)
  double* d_kpartials = nullptr;
  int kpart_stride = 0;
  double* d_kresult = nullptr;
  double* h_kresult = nullptr;
  double2* d_kcoef = nullptr;
  double2* h_kcoef = nullptr;

  // canonical staging buffers on the device (2 x max_rhs x V x 24 doubles)
  double* d_stage[2] = {nullptr, nullptr};
  size_t stage_cap = 0;

  // workspace spinors keyed by slot
  std::map<int, gbc::Spinor> ws;

  // autotuned hopping-kernel shapes, keyed by (precision, mode, dagger, reduce, nrhs)
  std::map<long long, int> tuned;  // autotuner decisions (context.cu tuned_shape)
  bool autotune = true;
  bool use_graphs = true;  // CUDA-graph replay of CG iteration blocks (GBC_GRAPHS=0: off)
  std::string tune_log;
  std::string dev_tag;  // device name and compute capability, for the persistent tune cache

  // learned preconditioner (opaque, owned by precond.cu)
  void* precond = nullptr;
  // apply_meo applies the symmetric operator M_s instead of M~ (set for a GBC_SYS_SYM* solve)
  bool sym = false;
  // device scalars of the inner BiCGStab (bicgstab.cu), bisc_cap right-hand sides
  void* d_bisc = nullptr;
  int bisc_cap = 0;
  // per-right-hand-side device flags the stencil launches honour while set (HopArgs::active): the
  // inner BiCGStab points them at its scalars so that converged right-hand sides cost nothing
  const int* hop_active = nullptr;
  int hop_active_stride = 0;
  gbc::Spinor hop_aux{};  // the FP32 field of a RED_DOT_AUX stencil launch (set around the call)
  // second stream for the host copies of gbc_solve that overlap device work (created on first use)
  cudaStream_t copy_stream = nullptr;
};

namespace gbc {

// ---- workspace -----------------------------------------------------------------------------
Spinor& workspace(gbc_ctx* c, int slot, int prec, int nrhs);
Spinor sub(const Spinor& s, int r0, int n);  // view of right-hand sides r0..r0+n-1
void free_ctx_memory(gbc_ctx* c);
void ensure_prec(gbc_ctx* c, int prec);  // pack gauge/clover in this precision
void ensure_stage(gbc_ctx* c, int nrhs);
Red red(gbc_ctx* c);

// ---- operator blocks on device fields (all of precision prec) ------------------------------
// out(out_parity) = mode-epilogue of a * D'(in)
void hop(gbc_ctx* c, int prec, int out_parity, int mode, bool dag, double a, const Spinor& in, const Spinor& out,
         const Spinor* self, const void* clov, int reduce, double twist = 0.0);
// out_o = M~ in_o (dag: M~^dag); reduce => |out|^2 in red(c).result[0][rhs]
void apply_meo(gbc_ctx* c, int prec, bool dag, const Spinor& in, const Spinor& out, const Spinor& tmp_e, int reduce);
void apply_clover(gbc_ctx* c, int prec, int parity, bool inverse, const Spinor& in, const Spinor& out);
// out_o = M_s in_o (dag: M_s^dag), the symmetric operator; reduce => |out|^2 as apply_meo
void apply_seo(gbc_ctx* c, int prec, bool dag, const Spinor& in, const Spinor& out, const Spinor& tmp_e, int reduce);
void ensure_sym(gbc_ctx* c, int prec);  // pack A_oo^-1 in this precision
// routes apply_meo to the symmetric operator while it lives
struct SymScope {
  gbc_ctx* c;
  bool old;
  SymScope(gbc_ctx* c_, bool on) : c(c_), old(c_->sym) { c->sym = on; }
  ~SymScope() { c->sym = old; }
};
void sync(gbc_ctx* c);
double now();

// ---- no-allocation operator (noalloc.cu) ---------------------------------------------------------
// makes gbc_apply_meo_noalloc's static scratch exist on the current device (loads its module)
int noalloc_reserve();

// ---- learned preconditioner (precond.cu) ----------------------------------------------------
void precond_free(gbc_ctx* c);
// out ~= M~^-1 in (odd checkerboard fields, same precision, nrhs right-hand sides)
void precond_apply(gbc_ctx* c, const Spinor& in, const Spinor& out);
// layers of the loaded network and the channels of layer l (its output side when out)
int precond_layers(gbc_ctx* c);
int precond_channels(gbc_ctx* c, int l, bool out);

// ---- inner BiCGStab (bicgstab.cu) ----------------------------------------------------------------
struct InnerStats {
  std::vector<int> iters;
  std::vector<int> status;
  int reliable = 0;
};
// M~ x = b in the sloppy operator po with accumulator precision pa, relative target tol on the
// iterated residual, reliable updates at delta; active[r] == 0 leaves right-hand side r at x = 0
InnerStats bicgstab(gbc_ctx* c, int pa, int po, double tol, int maxit, double delta, const Spinor& x,
                    const Spinor& b, const std::vector<int>& active);

// one fused BiCGStab update x += alpha p + omega (r - alpha v), r -= alpha v + omega t with |r|^2
// and (r0, r) in red(c).result rows 0, 1, 2 (alpha_omega: re, im of alpha, then of omega, per
// right-hand side); the precision pairs the inner solver uses: (FP64, FP64), (FP32, FP32), (FP32, FP16)
void bicgstab_xr_update(gbc_ctx* c, int pa, int po, const double* alpha_omega, int n, const Spinor& x,
                        const Spinor& r, const Spinor& p, const Spinor& v, const Spinor& t, const Spinor& r0);

// ---- solvers (solvers.cu) -------------------------------------------------------------------
// FP64 defect correction of the shifted normal systems (M~^dag M~ + sigma_q) psi_q = chi, one per
// right-hand side q of psi (FP64, holding the initial guesses), the corrections from CG with
// per-right-hand-side shifts d_shift (device) in the sloppy operator precision; returns the CG
// iterations per shift, the final FP64 |chi - (M~^dag M~ + sigma_q) psi_q|^2 in rr and a status
std::vector<int> refine_shifted(gbc_ctx* c, int sloppy, const Spinor& chi, const double* d_shift,
                                const Spinor& psi, const std::vector<double>& rsd, int max_iter,
                                std::vector<double>& rr, std::vector<int>& status);
// after_export (optional) runs once the solution is in psi_canon on the context stream and before
// the final residual check, which only reads it: gbc_solve starts the copy to the host there
int solve_device(gbc_ctx* c, const gbc_solve_params* p, int nrhs, double* psi_canon, const double* chi_canon,
                 gbc_result* res, const std::function<void()>* after_export = nullptr);

}  // namespace gbc
