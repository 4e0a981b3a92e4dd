// Batched solves over independent lattices of different sizes (one right-hand side each).
//
// Every lattice keeps its own context (geometry, links, clover, workspaces).  The outer FP64
// defect correction runs per lattice; the inner reliable-update CGNE runs for all lattices in
// lock step, and each of its stencil applications is ONE launch over a work table of
// (lattice, 128-site block) pairs covering all lattices (hop_kernel_multi), so small lattices do
// not leave the GPU idle.  The inner iterations run as one launch per step, replayed from CUDA
// graphs in blocks of 4 iterations, or (GBC_PERSISTENT=1) as a persistent cooperative kernel
// (batch_persistent.cuh) that performs up to 256 iterations per launch and returns only for a
// reliable update or convergence.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "ctx.h"

struct gbc_batch {
  std::vector<gbc_ctx*> ctx;
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> saved;
  gbc::HopArgs* d_args = nullptr;  // [4][n]: (hop1, hop2) x (PLUS, MINUS)
  gbc::LatCg* d_lat = nullptr;     // [n]: inner CG state per lattice
  int2* d_work = nullptr;
  int nwork = 0;
  gbc::GridBar* d_bar = nullptr;     // grid barrier of the persistent kernel
  gbc::PersistLat* d_pl = nullptr;   // [n]: reliable-update trigger state per lattice
  int* d_pout = nullptr;             // iterations run by the last persistent launch
  std::string err;
};

namespace gbc {
namespace {

enum { B_X = 500, B_B, B_R, B_P, B_MP, B_MMP, B_TE, B_T1, B_TEH, B_XD, B_BD, B_RD, B_TD1, B_TD2, B_TED, B_RS, B_ES, B_RHS };

HopArgs make_args(gbc_ctx* c, int prec, int out_parity, int mode, double a, const Spinor& in, const Spinor& out,
                  const Spinor* self, const void* clov, double twist) {
  const PrecFields& f = c->pf[pidx(prec)];
  HopArgs h{};
  h.g = c->g;
  h.out_parity = out_parity;
  h.nrhs = 1;
  h.in = in.v;
  h.in_norm = in.norm;
  h.in_rhs_bytes = in.rhs_bytes;
  h.out = out.v;
  h.out_norm = out.norm;
  h.out_rhs_bytes = out.rhs_bytes;
  if (self) {
    h.self = self->v;
    h.self_norm = self->norm;
    h.self_rhs_bytes = self->rhs_bytes;
  }
  h.norm_rhs_stride = in.norm_rhs_stride;
  for (int m = 0; m < 4; ++m) {
    h.gauge_fwd[m] = f.gauge[out_parity][m];
    h.gauge_bwd[m] = f.gauge[1 - out_parity][m];
  }
  h.clov = clov;
  h.a = a;
  h.twist = twist;
  h.partials = c->d_partials;
  h.part_stride = c->part_stride;
  (void)mode;
  return h;
}

}  // namespace
}  // namespace gbc

using namespace gbc;

extern "C" {

int gbc_batch_create(gbc_batch** out, int n, gbc_ctx* const* ctxs) {
  if (!out || n < 1 || !ctxs) return GBC_ERR_ARGS;
  gbc_batch* b = new gbc_batch;
  for (int i = 0; i < n; ++i) {
    if (!ctxs[i] || !ctxs[i]->have_gauge) {
      delete b;
      return GBC_ERR_STATE;
    }
    b->ctx.push_back(ctxs[i]);
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&b->d_args, sizeof(HopArgs) * 4 * n) != cudaSuccess ||
      cudaMalloc(&b->d_lat, sizeof(LatCg) * n) != cudaSuccess || cudaMalloc(&b->d_bar, sizeof(GridBar)) != cudaSuccess ||
      cudaMalloc(&b->d_pl, sizeof(PersistLat) * n) != cudaSuccess || cudaMalloc(&b->d_pout, sizeof(int) * 2) != cudaSuccess) {
    gbc_batch_destroy(b);
    return GBC_ERR_CUDA;
  }
  // work table: every 128-site block of every lattice, largest lattices first
  std::vector<int2> work;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return b->ctx[x]->g.Vh > b->ctx[y]->g.Vh; });
  for (int i : order)
    for (int sb = 0; sb < (b->ctx[i]->g.Vh + 127) / 128; ++sb) work.push_back(make_int2(i, sb));
  b->nwork = (int)work.size();
  if (cudaMalloc(&b->d_work, sizeof(int2) * work.size()) != cudaSuccess ||
      cudaMemcpy(b->d_work, work.data(), sizeof(int2) * work.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    gbc_batch_destroy(b);
    return GBC_ERR_CUDA;
  }
  *out = b;
  return GBC_OK;
}

void gbc_batch_destroy(gbc_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->d_args) cudaFree(b->d_args);
  if (b->d_lat) cudaFree(b->d_lat);
  if (b->d_work) cudaFree(b->d_work);
  if (b->d_bar) cudaFree(b->d_bar);
  if (b->d_pl) cudaFree(b->d_pl);
  if (b->d_pout) cudaFree(b->d_pout);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Solve M~ psi_l = chi_l (odd sites, host canonical arrays) for every lattice l of the batch
// to the FP64 true relative residual p->rsd_target.  res[l] per lattice.
int gbc_batch_solve(gbc_batch* b, const gbc_solve_params* pp, double* const* psi, const double* const* chi,
                    gbc_result* res) {
  if (!b || !pp || !psi || !chi || !res) return GBC_ERR_ARGS;
  const int n = (int)b->ctx.size();
  gbc_solve_params p = *pp;
  if (!(p.rsd_target > 0)) p.rsd_target = 1e-10;
  if (p.max_iter <= 0) p.max_iter = 10000;
  if (!(p.delta > 0)) p.delta = 0.1;
  if (!(p.inner_tol > 0)) p.inner_tol = 1e-6;
  int sloppy = p.sloppy_precision ? p.sloppy_precision : b->ctx[0]->opts.sloppy_precision;
  const int D = PREC_DOUBLE, S = PREC_SINGLE;
  const int pa = sloppy == D ? D : S;
  cudaStream_t s = b->stream;
  std::vector<cudaStream_t> saved(n);
  for (int l = 0; l < n; ++l) {
    saved[l] = b->ctx[l]->stream;
    b->ctx[l]->stream = s;  // every launch of the batch on one stream
  }
  auto restore = [&]() {
    for (int l = 0; l < n; ++l) b->ctx[l]->stream = saved[l];
  };
  try {
    const double t0 = now();
    cudaEvent_t e0, e1;
    GBC_CUDA(cudaEventCreate(&e0));
    GBC_CUDA(cudaEventCreate(&e1));
    GBC_CUDA(cudaEventRecord(e0, s));
    const long long l0 = launch_count();
    for (auto* c : b->ctx) {
      ensure_prec(c, D);
      ensure_prec(c, sloppy);
      ensure_prec(c, S);
      ensure_stage(c, 1);
      if (c->pf[pidx(sloppy)].recon != b->ctx[0]->pf[pidx(sloppy)].recon)
        throw std::string("lattices of a batch need the same link reconstruction");
    }
    struct L {
      Spinor x, bd, rd, t1, t2, ted, rs, es, rhs, r, pv, mp, mmp, te, th1, teh;
      double bb = 0, rr = 0, prev_rr = HUGE_VAL;
      int done = 0, iters = 0, outer = 0, reliable = 0, status = GBC_OK;
    };
    std::vector<L> lat(n);
    for (int l = 0; l < n; ++l) {
      gbc_ctx* c = b->ctx[l];
      L& q = lat[l];
      q.x = sub(workspace(c, B_X, D, 1), 0, 1);
      q.bd = sub(workspace(c, B_B, D, 1), 0, 1);
      q.rd = sub(workspace(c, B_RD, D, 1), 0, 1);
      q.t1 = sub(workspace(c, B_TD1, D, 1), 0, 1);
      q.t2 = sub(workspace(c, B_TD2, D, 1), 0, 1);
      q.ted = sub(workspace(c, B_TED, D, 1), 0, 1);
      q.rs = sub(workspace(c, B_RS, pa, 1), 0, 1);
      q.es = sub(workspace(c, B_ES, pa, 1), 0, 1);
      q.rhs = sub(workspace(c, B_RHS, pa, 1), 0, 1);
      q.r = sub(workspace(c, B_R, pa, 1), 0, 1);
      q.th1 = sub(workspace(c, B_T1, pa, 1), 0, 1);
      q.teh = sub(workspace(c, B_TEH, pa, 1), 0, 1);
      q.pv = sub(workspace(c, B_P, sloppy, 1), 0, 1);
      q.mp = sub(workspace(c, B_MP, sloppy, 1), 0, 1);
      q.mmp = sub(workspace(c, B_MMP, sloppy, 1), 0, 1);
      q.te = sub(workspace(c, B_TE, sloppy, 1), 0, 1);
      GBC_CUDA(cudaMemcpyAsync(c->d_stage[0], chi[l], sizeof(double) * 24 * c->V, cudaMemcpyHostToDevice, s));
      import_spinor(c->g, c->d_stage[0], (size_t)c->V * 24, 1, q.bd, s);
      blas_zero(c->g, q.x, s);
      blas_norm2(c->g, q.bd, red(c), s);
      GBC_CUDA(cudaMemcpyAsync(&q.bb, c->d_result, sizeof(double), cudaMemcpyDeviceToHost, s));
    }
    GBC_CUDA(cudaStreamSynchronize(s));
    // stencil arguments of the four launches of one CGNE iteration, for every lattice
    std::vector<HopArgs> args(4 * n);
    for (int l = 0; l < n; ++l) {
      gbc_ctx* c = b->ctx[l];
      L& q = lat[l];
      const PrecFields& f = c->pf[pidx(sloppy)];
      const double tw = c->act.twisted ? c->act.twisted_m : 0.0;
      args[0 * n + l] = make_args(c, sloppy, 0, HOP_CLOV, 1.0, q.pv, q.te, nullptr, f.clovinv, 0.0);
      args[1 * n + l] = make_args(c, sloppy, 1, HOP_XPAY, -0.25, q.te, q.mp, &q.pv, f.clov[1], tw);
      args[2 * n + l] = make_args(c, sloppy, 0, HOP_CLOV, 1.0, q.mp, q.te, nullptr, f.clovinv, 0.0);
      args[3 * n + l] = make_args(c, sloppy, 1, HOP_XPAY, -0.25, q.te, q.mmp, &q.mp, f.clov[1], tw);
    }
    GBC_CUDA(cudaMemcpyAsync(b->d_args, args.data(), sizeof(HopArgs) * 4 * n, cudaMemcpyHostToDevice, s));
    const int recon = b->ctx[0]->pf[pidx(sloppy)].recon;
    // GBC_PERSISTENT=1: the inner iterations as one persistent kernel per block of iterations.
    // The default is one launch per step replayed from CUDA graphs: on GB300 it matches the
    // persistent kernel on a batch of 33 work items and is 10 % faster on one of 1956 (its kernel
    // boundaries cost less than the persistent kernel's 5 software grid barriers per iteration).
    const char* pe = getenv("GBC_PERSISTENT");
    bool persist = pe && pe[0] == '1' && n <= kPersistMaxLattices && pa == S && sloppy != D;
    auto multi = [&](int k, int mode, bool dag, bool reduce) {
      if (hop_multi_launch(sloppy, recon, mode, dag, reduce, b->d_args + k * n, b->d_work, b->nwork, s) < 0)
        throw std::string("multi-lattice kernel variant not compiled");
      count_launch();
    };
    // the inner CG state of every lattice, for the multi-lattice BLAS and scalar kernels; the
    // stencil's |M~ p|^2 partials land in row 0 of each context's partials, the update's in row 1
    std::vector<LatCg> lc(n);
    for (int l = 0; l < n; ++l) {
      gbc_ctx* c = b->ctx[l];
      L& q = lat[l];
      lc[l] = LatCg{c->g.Vh, (c->g.Vh + 127) / 128, q.es, q.r, q.pv, q.mmp, c->d_cg, c->d_partials,
                    c->d_partials + c->part_stride};
    }
    GBC_CUDA(cudaMemcpyAsync(b->d_lat, lc.data(), sizeof(LatCg) * n, cudaMemcpyHostToDevice, s));
    // one CGNE iteration for every lattice in 8 launches: M~ p (two stencil launches), alpha,
    // M~^dag (two), the fused update with |r|^2, beta, p = r + b p
    auto body = [&]() {
      multi(0, HOP_CLOV, false, false);
      multi(1, HOP_XPAY, false, true);
      batch_cg_alpha(b->d_lat, n, s);
      multi(2, HOP_CLOV, true, false);
      multi(3, HOP_XPAY, true, false);
      batch_cg_update(pa, sloppy, b->d_lat, b->d_work, b->nwork, s);
      batch_cg_beta(b->d_lat, n, s);
      batch_xpay(pa, sloppy, b->d_lat, b->d_work, b->nwork, s);
    };
    int total = 0;
    for (int outer = 0; outer <= 50; ++outer) {
      // FP64 residual per lattice
      bool all = true;
      double worst = 0;
      for (int l = 0; l < n; ++l) {
        gbc_ctx* c = b->ctx[l];
        L& q = lat[l];
        if (q.done) continue;
        apply_meo(c, D, false, q.x, q.t1, q.ted, false);
        blas_xmy_norm2(c->g, q.bd, q.t1, red(c), s);  // t1 = b - M x
        GBC_CUDA(cudaMemcpyAsync(&q.rr, c->d_result, sizeof(double), cudaMemcpyDeviceToHost, s));
      }
      GBC_CUDA(cudaStreamSynchronize(s));
      for (int l = 0; l < n; ++l) {
        L& q = lat[l];
        if (q.done) continue;
        if (std::isfinite(q.prev_rr) && !(q.rr <= q.prev_rr)) {
          // the last correction left the FP64 residual larger (an inner solve that broke down):
          // take it back and stop this lattice with the better iterate
          gbc_ctx* c = b->ctx[l];
          c->h_coef[0] = make_double2(-1.0, 0.0);
          c->h_coef[1] = make_double2(1.0, 0.0);
          GBC_CUDA(cudaMemcpyAsync(c->d_ca, c->h_coef, sizeof(double2), cudaMemcpyHostToDevice, s));
          GBC_CUDA(cudaMemcpyAsync(c->d_cb, c->h_coef + 1, sizeof(double2), cudaMemcpyHostToDevice, s));
          blas_axpby(c->g, c->d_ca, q.es, c->d_cb, q.x, s);
          GBC_CUDA(cudaStreamSynchronize(s));
          q.rr = q.prev_rr;
          q.status = GBC_ERR_NOT_CONVERGED;
          q.done = 1;
          continue;
        }
        if (!std::isfinite(q.rr)) {
          q.status = GBC_ERR_NONFINITE;
          q.done = 1;
          continue;
        }
        q.prev_rr = q.rr;
        if (q.rr <= p.rsd_target * p.rsd_target * q.bb) q.done = 1;
        else {
          all = false;
          worst = std::max(worst, std::sqrt(q.rr / q.bb));
        }
      }
      if (all || outer == 50 || total >= p.max_iter) break;
      const double itol = std::min(0.1, std::max(p.inner_tol, 0.5 * p.rsd_target / worst));
      // inner right-hand sides rhs = M~^dag r (accumulator precision), CG state per lattice
      std::vector<double> rr0(n, 0.0), bn(n, 0.0);
      for (int l = 0; l < n; ++l) {
        gbc_ctx* c = b->ctx[l];
        L& q = lat[l];
        ++q.outer;
        blas_copy(c->g, q.rs, q.t1, s);
        apply_meo(c, pa, true, q.rs, q.rhs, q.teh, false);
        blas_zero(c->g, q.es, s);
        blas_copy(c->g, q.r, q.rhs, s);
        blas_copy(c->g, q.pv, q.r, s);
        blas_norm2(c->g, q.r, red(c), s);
        GBC_CUDA(cudaMemcpyAsync(&rr0[l], c->d_result, sizeof(double), cudaMemcpyDeviceToHost, s));
      }
      GBC_CUDA(cudaStreamSynchronize(s));
      std::vector<double> maxrr(n), at_update(n), last_nr(n, HUGE_VAL);
      std::vector<int> stall(n, 0);
      for (int l = 0; l < n; ++l) {
        L& q = lat[l];
        CGScalars st{};
        st.c = st.cp = st.c_prev = rr0[l];
        st.rsd_sq = itol * itol * rr0[l];
        st.active = !q.done && rr0[l] > 0;
        maxrr[l] = at_update[l] = std::sqrt(rr0[l]);
        GBC_CUDA(cudaMemcpyAsync(b->ctx[l]->d_cg, &st, sizeof(CGScalars), cudaMemcpyHostToDevice, s));
      }
      GBC_CUDA(cudaStreamSynchronize(s));
      // The persistent kernel runs up to kPersistIters iterations per launch and stops by itself
      // for a reliable update; otherwise the first iteration runs uncaptured, then graph blocks.
      constexpr int kBlock = 4;
      constexpr int kPersistIters = 256;
      cudaGraphExec_t exec = nullptr;
      long long gl = 0;
      int k = 0;
      bool any = true;
      while (any && k < p.max_iter) {
        bool ran = false;
        if (persist) {
          std::vector<PersistLat> hp(n);
          for (int l = 0; l < n; ++l) hp[l] = PersistLat{maxrr[l], at_update[l]};
          GBC_CUDA(cudaMemcpyAsync(b->d_pl, hp.data(), sizeof(PersistLat) * n, cudaMemcpyHostToDevice, s));
          const int kmax = std::min(kPersistIters, p.max_iter - k);
          const int r = batch_cg_persistent(pa, sloppy, recon, b->d_args, b->d_lat, b->d_work, b->nwork, n, kmax,
                                            p.delta, b->d_pl, b->d_bar, b->d_pout, s);
          if (r > 0) GBC_CUDA((cudaError_t)r);
          if (r < 0) {
            persist = false;  // no persistent variant, or the cooperative launch was refused
          } else {
            GridBar hb{};
            int ran_iters = 0;
            GBC_CUDA(cudaMemcpyAsync(&hb, b->d_bar, sizeof(GridBar), cudaMemcpyDeviceToHost, s));
            GBC_CUDA(cudaMemcpyAsync(&ran_iters, b->d_pout, sizeof(int), cudaMemcpyDeviceToHost, s));
            GBC_CUDA(cudaMemcpyAsync(hp.data(), b->d_pl, sizeof(PersistLat) * n, cudaMemcpyDeviceToHost, s));
            GBC_CUDA(cudaStreamSynchronize(s));
            if (hb.err) {
              if (exec) cudaGraphExecDestroy(exec);
              throw std::string("persistent batch kernel: a grid-barrier wait gave up at barrier ") +
                  std::to_string(hb.where);
            }
            for (int l = 0; l < n; ++l) maxrr[l] = hp[l].maxrr;
            k += ran_iters;
            ran = true;
          }
        }
        if (ran) {
        } else if (k > 0 && b->ctx[0]->use_graphs) {
          if (!exec) {
            cudaGraph_t graph;
            const long long c0 = launch_count();
            GBC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            for (int q = 0; q < kBlock; ++q) body();
            GBC_CUDA(cudaStreamEndCapture(s, &graph));
            GBC_CUDA(cudaGraphInstantiate(&exec, graph, 0));
            cudaGraphDestroy(graph);
            gl = launch_count() - c0;
            count_launch(-gl);
          }
          GBC_CUDA(cudaGraphLaunch(exec, s));
          count_launch(gl);
          k += kBlock;
        } else {
          body();
          k += 1;
        }
        std::vector<CGScalars> hs(n);
        for (int l = 0; l < n; ++l)
          GBC_CUDA(cudaMemcpyAsync(&hs[l], b->ctx[l]->d_cg, sizeof(CGScalars), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        any = false;
        bool trigger = false;
        for (int l = 0; l < n; ++l) {
          if (!hs[l].active) continue;
          any = true;
          const double rn = std::sqrt(hs[l].cp);
          maxrr[l] = std::max(maxrr[l], rn);
          if (rn < p.delta * maxrr[l]) trigger = true;
          if (rn > at_update[l]) trigger = true;  // the recurrence drifted up: check the true residual
        }
        if (any && trigger) {
          // reliable update for every active lattice: r = rhs - M~^dag M~ e (accumulator precision)
          std::vector<double> nr(n, 0.0);
          for (int l = 0; l < n; ++l) {
            gbc_ctx* c = b->ctx[l];
            L& q = lat[l];
            if (!hs[l].active) continue;
            ++q.reliable;
            apply_meo(c, pa, false, q.es, q.th1, q.teh, false);
            apply_meo(c, pa, true, q.th1, q.r, q.teh, false);
            blas_xmy_norm2(c->g, q.rhs, q.r, red(c), s);
            GBC_CUDA(cudaMemcpyAsync(&nr[l], c->d_result, sizeof(double), cudaMemcpyDeviceToHost, s));
          }
          GBC_CUDA(cudaStreamSynchronize(s));
          for (int l = 0; l < n; ++l) {
            if (!hs[l].active) continue;
            hs[l].c = hs[l].cp = nr[l];
            maxrr[l] = at_update[l] = std::sqrt(nr[l]);
            // three reliable updates in a row that fail to halve the true residual: the accumulator
            // precision's floor is reached, the FP64 outer loop takes over
            stall[l] = nr[l] > 0.25 * last_nr[l] ? stall[l] + 1 : 0;
            last_nr[l] = nr[l];
            if (!(nr[l] > hs[l].rsd_sq) || stall[l] >= 3) {
              hs[l].active = 0;
              hs[l].b = 0;
            }
            GBC_CUDA(cudaMemcpyAsync(b->ctx[l]->d_cg, &hs[l], sizeof(CGScalars), cudaMemcpyHostToDevice, s));
          }
          GBC_CUDA(cudaStreamSynchronize(s));
        }
      }
      if (exec) cudaGraphExecDestroy(exec);
      int mx = 0;
      for (int l = 0; l < n; ++l) {
        gbc_ctx* c = b->ctx[l];
        L& q = lat[l];
        CGScalars hs{};
        GBC_CUDA(cudaMemcpyAsync(&hs, c->d_cg, sizeof(CGScalars), cudaMemcpyDeviceToHost, s));
        GBC_CUDA(cudaStreamSynchronize(s));
        if (!q.done) {
          q.iters += hs.iters;
          mx = std::max(mx, hs.iters);
          blas_xpy(c->g, q.x, q.es, s);
        }
      }
      total += mx;
    }
    GBC_CUDA(cudaEventRecord(e1, s));
    for (int l = 0; l < n; ++l) {
      gbc_ctx* c = b->ctx[l];
      L& q = lat[l];
      GBC_CUDA(cudaMemcpyAsync(c->d_stage[1], psi[l], sizeof(double) * 24 * c->V, cudaMemcpyHostToDevice, s));
      export_spinor(c->g, c->d_stage[1], (size_t)c->V * 24, 1, q.x, s);
      GBC_CUDA(cudaMemcpyAsync(psi[l], c->d_stage[1], sizeof(double) * 24 * c->V, cudaMemcpyDeviceToHost, s));
    }
    GBC_CUDA(cudaStreamSynchronize(s));
    float ms = 0;
    GBC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double t1 = now();
    int worst = GBC_OK;
    for (int l = 0; l < n; ++l) {
      L& q = lat[l];
      gbc_result& o = res[l];
      std::memset(&o, 0, sizeof(o));
      o.n_count = q.iters;
      o.n_outer = q.outer;
      o.n_reliable = q.reliable;
      o.resid = std::sqrt(q.rr);
      o.rel_resid = q.bb > 0 ? std::sqrt(q.rr / q.bb) : o.resid;
      o.status = q.status != GBC_OK ? q.status : (q.done ? GBC_OK : GBC_ERR_NOT_CONVERGED);
      o.seconds = t1 - t0;
      o.device_seconds = ms * 1e-3;
      o.launches = launch_count() - l0;
      if (o.status != GBC_OK && worst == GBC_OK) worst = o.status;
    }
    restore();
    return worst;
  } catch (const CudaError& e) {
    restore();
    b->err = std::string(e.where) + ": " + cudaGetErrorString(e.e);
    return GBC_ERR_CUDA;
  } catch (const std::string& m) {
    restore();
    b->err = m;
    return GBC_ERR_STATE;
  }
}

const char* gbc_batch_last_error(gbc_batch* b) { return b ? b->err.c_str() : ""; }

}  // extern "C"
