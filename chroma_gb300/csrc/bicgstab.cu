// BiCGStab on M~ x = b, batched over right-hand sides, as the inner solver of the FP64 defect
// correction (GBC_SOLVER_BICGSTAB; QUDA's BICGSTAB SolverType of the clover solver XML,
// lib/actions/ferm/invert/quda_solvers/enum_quda_io.h:21-27, syssolver_linop_clover_quda_w.h:257-259).
//
//   v = A p;  alpha = rho / (r0, v);  s = r - alpha v;  t = A s;  omega = (t, s) / (t, t)
//   x += alpha p + omega s;  r = s - omega t;  rho' = (r0, r);  beta = (rho' / rho)(alpha / omega)
//   p = r + beta (p - omega v)
//
// The operator and the vectors it reads (p, v, s, t) are in the sloppy precision; x, r and the
// shadow residual r0 in the accumulator precision (an fp16 r0 made the iteration counts of the
// right-hand sides spread and cost more reliable updates than its bandwidth saved).  x and r are
// updated from the accumulator-precision r of the step before (x += alpha p + omega (r - alpha v),
// r -= alpha v + omega t), so the sloppy copy of s only feeds the operator and the (t, s) product,
// which the stencil launch that writes t sums in its epilogue.  Every scalar lives on the device
// (one thread per right-hand side), so iterations replay from CUDA graphs; the host looks at the
// scalars every few iterations for reliable updates (r = b - A x with the accumulator-precision
// operator), for stalls at the accumulator precision's floor, and for convergence.  A right-hand
// side that has converged is skipped by every kernel of the iteration (its device flag), so the
// batch's slowest sources do not make the others pay.
#include <cmath>
#include <cstring>

#include "ctx.h"
#include "gbc_device.cuh"

namespace gbc {

struct BiScal {
  double2 rho, alpha, omega, beta;
  double rr, rsd_sq;
  int active, iters, status;
};

namespace {

constexpr int BT = 256;

__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <typename P>
__device__ __forceinline__ void ldv(cplx<typename P::real> (&x)[12], const Spinor& f, int idx, int r) {
  load_spinor<P>(x, (const char*)f.v + (size_t)r * f.rhs_bytes, f.norm ? f.norm + (size_t)r * f.norm_rhs_stride : nullptr,
                 idx, f.stride);
}
template <typename P>
__device__ __forceinline__ void stv(const Spinor& f, int idx, int r, const cplx<typename P::real> (&x)[12]) {
  store_spinor<P>((char*)f.v + (size_t)r * f.rhs_bytes, f.norm ? f.norm + (size_t)r * f.norm_rhs_stride : nullptr, idx,
                  f.stride, x);
}

// complex components 4c .. 4c + 3 of right-hand side r at site idx; n = the site norm of an fp16
// field (ignored otherwise)
template <typename P>
__device__ __forceinline__ void ld4(cplx<typename P::real> (&x)[4], const Spinor& f, int idx, int r, int c, float n) {
  const char* base = (const char*)f.v + (size_t)r * f.rhs_bytes;
  if constexpr (std::is_same<P, PrecD>::value) {
    const double2* p = reinterpret_cast<const double2*>(base);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double2 v = ldg(p + (size_t)(4 * c + q) * f.stride + idx);
      x[q] = {v.x, v.y};
    }
  } else if constexpr (std::is_same<P, PrecS>::value) {
    const float4* p = reinterpret_cast<const float4*>(base);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float4 v = ldg(p + (size_t)(2 * c + h) * f.stride + idx);
      x[2 * h] = {v.x, v.y};
      x[2 * h + 1] = {v.z, v.w};
    }
  } else {
    const uint4 v = ldg(reinterpret_cast<const uint4*>(base) + (size_t)c * f.stride + idx);
    const float2 a = h2f(v.x), b = h2f(v.y), d = h2f(v.z), e = h2f(v.w);
    x[0] = {a.x * n, a.y * n};
    x[1] = {b.x * n, b.y * n};
    x[2] = {d.x * n, d.y * n};
    x[3] = {e.x * n, e.y * n};
  }
}
// store components 4c .. 4c + 3 (FP64 / FP32 fields only: an fp16 site needs all 12 for its norm)
template <typename P>
__device__ __forceinline__ void st4(const Spinor& f, int idx, int r, int c, const cplx<typename P::real> (&x)[4]) {
  static_assert(!std::is_same<P, PrecH>::value, "fp16 stores go through store_spinor");
  char* base = (char*)f.v + (size_t)r * f.rhs_bytes;
  if constexpr (std::is_same<P, PrecD>::value) {
    double2* p = reinterpret_cast<double2*>(base);
#pragma unroll
    for (int q = 0; q < 4; ++q) p[(size_t)(4 * c + q) * f.stride + idx] = make_double2(x[q].re, x[q].im);
  } else {
    float4* p = reinterpret_cast<float4*>(base);
#pragma unroll
    for (int h = 0; h < 2; ++h)
      p[(size_t)(2 * c + h) * f.stride + idx] = make_float4(x[2 * h].re, x[2 * h].im, x[2 * h + 1].re, x[2 * h + 1].im);
  }
}
template <typename P>
__device__ __forceinline__ float site_norm(const Spinor& f, int idx, int r) {
  if constexpr (std::is_same<P, PrecH>::value) return ldg(f.norm + (size_t)r * f.norm_rhs_stride + idx);
  return 1.0f;
}

// grid-stride site loop, one y-block row per right-hand side, NRED sums per right-hand side
// F::kMinb resident blocks per SM: 4 (64 registers) for the FP32 accumulators, 2 for FP64
// A right-hand side that has converged (sc[r].active == 0) is skipped: its vectors are frozen and
// its partial rows are never read.
template <int NRED, class F>
__global__ void __launch_bounds__(BT, F::kMinb) bi_site_kernel(int Vh, F f, const BiScal* sc, double* partials,
                                                               int part_stride, int nrhs) {
  using A = typename AccOf<F>::type;  // thread and warp sums in the compute precision
  const int r = blockIdx.y;
  if (!sc[r].active) return;  // uniform over the block
  A acc[NRED > 0 ? NRED : 1];
#pragma unroll
  for (int q = 0; q < (NRED > 0 ? NRED : 1); ++q) acc[q] = 0;
  for (int idx = blockIdx.x * BT + threadIdx.x; idx < Vh; idx += gridDim.x * BT) f(idx, r, acc);
  if constexpr (NRED > 0) {
    __shared__ double sh[NRED][BT / 32];
#pragma unroll
    for (int q = 0; q < NRED; ++q) {
      A v = acc[q];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if ((threadIdx.x & 31) == 0) sh[q][threadIdx.x >> 5] = (double)v;
    }
    __syncthreads();
    if (threadIdx.x < NRED) {
      double s = 0.0;
#pragma unroll
      for (int w = 0; w < BT / 32; ++w) s += sh[threadIdx.x][w];
      partials[((size_t)threadIdx.x * nrhs + r) * part_stride + blockIdx.x] = s;
    }
  }
}

// s = r - alpha v
template <typename PA, typename PO>
struct SUpdF {
  static constexpr int kMinb = std::is_same<PA, PrecD>::value ? 2 : 4;
  const BiScal* sc;
  Spinor r, v, s;
  __device__ void operator()(int idx, int k, double*) const {
    using T = typename PO::real;
    cplx<typename PA::real> rs[12];
    cplx<T> vs[12], ss[12];
    ldv<PA>(rs, r, idx, k);
    ldv<PO>(vs, v, idx, k);
    const double2 al = sc[k].alpha;
    const cplx<T> a{(T)al.x, (T)al.y};
#pragma unroll
    for (int q = 0; q < 12; ++q) ss[q] = cplx<T>{(T)rs[q].re, (T)rs[q].im} - a * vs[q];
    stv<PO>(s, idx, k, ss);
  }
};

// (t, s) and |t|^2
template <typename PO>
struct TsTtF {
  static constexpr int kMinb = std::is_same<PO, PrecD>::value ? 2 : 4;
  using Acc = typename PO::real;
  Spinor t, s;
  __device__ void operator()(int idx, int k, Acc* acc) const {
    using T = typename PO::real;
    cplx<T> ts[12], ss[12];
    ldv<PO>(ts, t, idx, k);
    ldv<PO>(ss, s, idx, k);
    T re = 0, im = 0, tt = 0;
#pragma unroll
    for (int q = 0; q < 12; ++q) {
      re = fmadd(ts[q].re, ss[q].re, fmadd(ts[q].im, ss[q].im, re));
      im = fmadd(ts[q].re, ss[q].im, fmadd(-ts[q].im, ss[q].re, im));
      tt = fmadd(ts[q].re, ts[q].re, fmadd(ts[q].im, ts[q].im, tt));
    }
    acc[0] += re;
    acc[1] += im;
    acc[2] += tt;
  }
};

// x += alpha p + omega (r - alpha v);  r -= alpha v + omega t;  |r|^2 and (r0, r).  Six vectors
// in and two out per site: processed four colour-spin components at a time (a whole site of all
// eight would hold ~150 registers and leave one block per SM for a bandwidth-bound loop).
template <typename PA, typename PO>
struct XRUpdF {
  static constexpr int kMinb = std::is_same<PA, PrecD>::value ? 2 : 4;
  using Acc = typename PA::real;
  const BiScal* sc;
  Spinor x, r, p, v, t, r0;
  __device__ void operator()(int idx, int k, Acc* acc) const {
    using T = typename PA::real;
    using U = typename PO::real;
    const float np = site_norm<PO>(p, idx, k), nv = site_norm<PO>(v, idx, k), nt = site_norm<PO>(t, idx, k);
    const float nh = site_norm<PA>(r0, idx, k);
    const double2 al = sc[k].alpha, om = sc[k].omega;
    const cplx<T> a{(T)al.x, (T)al.y}, w{(T)om.x, (T)om.y};
    T rr = 0, re = 0, im = 0;
#pragma unroll 1
    for (int c = 0; c < 3; ++c) {
      cplx<T> xs[4], rs[4], hs[4];
      cplx<U> ps[4], vs[4], ts[4];
      ld4<PA>(xs, x, idx, k, c, 1.f);
      ld4<PA>(rs, r, idx, k, c, 1.f);
      ld4<PA>(hs, r0, idx, k, c, nh);
      ld4<PO>(ps, p, idx, k, c, np);
      ld4<PO>(vs, v, idx, k, c, nv);
      ld4<PO>(ts, t, idx, k, c, nt);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const cplx<T> pq{(T)ps[q].re, (T)ps[q].im}, vq{(T)vs[q].re, (T)vs[q].im}, tq{(T)ts[q].re, (T)ts[q].im};
        const cplx<T> hq = hs[q];
        const cplx<T> sq = rs[q] - a * vq;
        xs[q] = xs[q] + a * pq + w * sq;
        rs[q] = sq - w * tq;
        rr = fmadd(rs[q].re, rs[q].re, fmadd(rs[q].im, rs[q].im, rr));
        re = fmadd(hq.re, rs[q].re, fmadd(hq.im, rs[q].im, re));
        im = fmadd(hq.re, rs[q].im, fmadd(-hq.im, rs[q].re, im));
      }
      st4<PA>(x, idx, k, c, xs);
      st4<PA>(r, idx, k, c, rs);
    }
    acc[0] += rr;
    acc[1] += re;
    acc[2] += im;
  }
};

// p = r + beta (p - omega v)
template <typename PA, typename PO>
struct PUpdF {
  static constexpr int kMinb = std::is_same<PA, PrecD>::value ? 2 : 4;
  const BiScal* sc;
  Spinor r, p, v;
  __device__ void operator()(int idx, int k, double*) const {
    using T = typename PO::real;
    cplx<typename PA::real> rs[12];
    cplx<T> ps[12], vs[12];
    ldv<PA>(rs, r, idx, k);
    ldv<PO>(ps, p, idx, k);
    ldv<PO>(vs, v, idx, k);
    const double2 be = sc[k].beta, om = sc[k].omega;
    const cplx<T> b{(T)be.x, (T)be.y}, w{(T)om.x, (T)om.y};
#pragma unroll
    for (int q = 0; q < 12; ++q) ps[q] = cplx<T>{(T)rs[q].re, (T)rs[q].im} + b * (ps[q] - w * vs[q]);
    stv<PO>(p, idx, k, ps);
  }
};

// alpha = rho / (r0, v)          res = [Re, Im][n]
__global__ void bi_alpha(BiScal* sc, const double* res, int n) {
  const int k = threadIdx.x;
  if (k >= n) return;
  BiScal q = sc[k];
  q.alpha = make_double2(0.0, 0.0);
  if (q.active) {
    const double2 d = make_double2(res[k], res[n + k]);
    if (d.x * d.x + d.y * d.y > 0.0 && std::isfinite(d.x) && std::isfinite(d.y)) {
      q.alpha = cdiv(q.rho, d);
    } else {
      q.active = 0;
      q.status = GBC_ERR_BREAKDOWN;
    }
  }
  sc[k] = q;
}

// omega = (t, s) / (t, t)         res = [Re ts, Im ts, tt][n]
__global__ void bi_omega(BiScal* sc, const double* res, int n) {
  const int k = threadIdx.x;
  if (k >= n) return;
  BiScal q = sc[k];
  const double tt = res[2 * n + k];
  q.omega = (q.active && tt > 0.0) ? make_double2(res[k] / tt, res[n + k] / tt) : make_double2(0.0, 0.0);
  sc[k] = q;
}

// |r|^2, rho' = (r0, r); converged -> inactive; beta = (rho'/rho)(alpha/omega)   res = [rr, Re, Im][n]
__global__ void bi_beta(BiScal* sc, const double* res, int n) {
  const int k = threadIdx.x;
  if (k >= n) return;
  BiScal q = sc[k];
  q.beta = make_double2(0.0, 0.0);
  if (q.active) {
    q.iters += 1;
    q.rr = res[k];
    const double2 rho1 = make_double2(res[n + k], res[2 * n + k]);
    if (!std::isfinite(q.rr)) {
      q.active = 0;
      q.status = GBC_ERR_NONFINITE;
    } else if (!(q.rr > q.rsd_sq)) {
      q.active = 0;  // converged
    } else if (q.omega.x == 0.0 && q.omega.y == 0.0) {
      q.active = 0;
      q.status = GBC_ERR_BREAKDOWN;
    } else {
      q.beta = cmul(cdiv(rho1, q.rho), cdiv(q.alpha, q.omega));
    }
    q.rho = rho1;
  }
  sc[k] = q;
}

template <int NRED, class F>
void run(gbc_ctx* c, int nrhs, const BiScal* sc, const F& f) {
  const Geom& g = c->g;
  dim3 grid(blas_blocks(g), nrhs);
  const Red rd = red(c);
  bi_site_kernel<NRED, F><<<grid, BT, 0, c->stream>>>(g.Vh, f, sc, rd.partials, rd.part_stride, nrhs);
  count_launch();
  if (NRED > 0) reduce_finalize(rd, NRED, nrhs, grid.x, c->stream);
}

template <typename PA, typename PO>
void iteration(gbc_ctx* c, int po, BiScal* sc, int n, const Spinor& x, const Spinor& r, const Spinor& r0,
               const Spinor& p, const Spinor& v, const Spinor& s, const Spinor& t, const Spinor& te) {
  cudaStream_t st = c->stream;
  const int nth = ((n + 31) / 32) * 32;  // one thread per right-hand side
  if (!c->sym && r0.prec == PREC_SINGLE) {
    // (r0, v) summed in the epilogue of the stencil launch that writes v = M~ p (r0 at its sites)
    c->hop_aux = r0;
    apply_meo(c, po, false, p, v, te, RED_DOT_AUX);
    c->hop_aux = Spinor{};
  } else {
    apply_meo(c, po, false, p, v, te, RED_NONE);
    blas_cdot(c->g, r0, v, red(c), st);
  }
  bi_alpha<<<1, nth, 0, st>>>(sc, c->d_result, n);
  count_launch();
  run<0>(c, n, sc, SUpdF<PA, PO>{sc, r, v, s});
  if (c->sym) {
    apply_meo(c, po, false, s, t, te, RED_NONE);
    run<3>(c, n, sc, TsTtF<PO>{t, s});
  } else {
    // (t, s) and (t, t) summed in the epilogue of the stencil launch that writes t (s is its self)
    apply_meo(c, po, false, s, t, te, RED_DOT_SELF);
  }
  bi_omega<<<1, nth, 0, st>>>(sc, c->d_result, n);
  count_launch();
  run<3>(c, n, sc, XRUpdF<PA, PO>{sc, x, r, p, v, t, r0});
  bi_beta<<<1, nth, 0, st>>>(sc, c->d_result, n);
  count_launch();
  run<0>(c, n, sc, PUpdF<PA, PO>{sc, r, p, v});
}

}  // namespace

void bicgstab_xr_update(gbc_ctx* c, int pa, int po, const double* alpha_omega, int n, const Spinor& x,
                        const Spinor& r, const Spinor& p, const Spinor& v, const Spinor& t, const Spinor& r0) {
  if (!((pa == PREC_DOUBLE && po == PREC_DOUBLE) || (pa == PREC_SINGLE && (po == PREC_SINGLE || po == PREC_HALF))))
    throw std::string("BiCGStab update not built for this precision pair");
  if (c->bisc_cap < n) {
    if (c->d_bisc) cudaFree(c->d_bisc);
    c->d_bisc = nullptr;
    c->bisc_cap = 0;
    GBC_CUDA(cudaMalloc(&c->d_bisc, sizeof(BiScal) * n));
    c->bisc_cap = n;
  }
  BiScal* d_sc = static_cast<BiScal*>(c->d_bisc);
  std::vector<BiScal> hs(n);
  for (int i = 0; i < n; ++i) {
    std::memset(&hs[i], 0, sizeof(BiScal));
    hs[i].alpha = make_double2(alpha_omega[4 * i], alpha_omega[4 * i + 1]);
    hs[i].omega = make_double2(alpha_omega[4 * i + 2], alpha_omega[4 * i + 3]);
    hs[i].active = 1;
  }
  GBC_CUDA(cudaMemcpyAsync(d_sc, hs.data(), sizeof(BiScal) * n, cudaMemcpyHostToDevice, c->stream));
  if (pa == PREC_DOUBLE) run<3>(c, n, d_sc, XRUpdF<PrecD, PrecD>{d_sc, x, r, p, v, t, r0});
  else if (po == PREC_SINGLE) run<3>(c, n, d_sc, XRUpdF<PrecS, PrecS>{d_sc, x, r, p, v, t, r0});
  else run<3>(c, n, d_sc, XRUpdF<PrecS, PrecH>{d_sc, x, r, p, v, t, r0});
  GBC_CUDA(cudaGetLastError());
  sync(c);  // hs goes out of scope
}

InnerStats bicgstab(gbc_ctx* c, int pa, int po, double tol, int maxit, double delta, const Spinor& x,
                    const Spinor& b, const std::vector<int>& active) {
  const int n = x.nrhs;
  const Geom& g = c->g;
  cudaStream_t st = c->stream;
  enum { S_R = 600, S_R0, S_P, S_V, S_S, S_T, S_TE, S_TA, S_TEA };
  Spinor r = sub(workspace(c, S_R + 20 * pidx(pa), pa, n), 0, n);
  Spinor r0 = sub(workspace(c, S_R0 + 20 * pidx(pa), pa, n), 0, n);
  Spinor p = sub(workspace(c, S_P + 20 * pidx(po), po, n), 0, n);
  Spinor v = sub(workspace(c, S_V + 20 * pidx(po), po, n), 0, n);
  Spinor s = sub(workspace(c, S_S + 20 * pidx(po), po, n), 0, n);
  Spinor t = sub(workspace(c, S_T + 20 * pidx(po), po, n), 0, n);
  Spinor te = sub(workspace(c, S_TE + 20 * pidx(po), po, n), 0, n);
  InnerStats out;
  out.iters.assign(n, 0);
  out.status.assign(n, GBC_OK);

  // x = 0, r = r0 = p = b
  blas_zero(g, x, st);
  blas_copy(g, r, b, st);
  blas_copy(g, r0, b, st);
  blas_copy(g, p, b, st);
  blas_norm2(g, b, red(c), st);
  std::vector<double> bb(n), rho0(2 * n);
  GBC_CUDA(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  sync(c);
  std::memcpy(bb.data(), c->h_result, sizeof(double) * n);
  blas_cdot(g, r0, r, red(c), st);  // rho = (r0, r)
  GBC_CUDA(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st));
  sync(c);
  std::memcpy(rho0.data(), c->h_result, sizeof(double) * 2 * n);

  // device scalars: kept in the context (no allocation inside the outer loop)
  if (c->bisc_cap < n) {
    if (c->d_bisc) cudaFree(c->d_bisc);
    c->d_bisc = nullptr;
    c->bisc_cap = 0;
    GBC_CUDA(cudaMalloc(&c->d_bisc, sizeof(BiScal) * n));
    c->bisc_cap = n;
  }
  BiScal* d_sc = static_cast<BiScal*>(c->d_bisc);
  std::vector<BiScal> hs(n);
  std::vector<double> maxr(n), last_nr(n, HUGE_VAL), at_update(n);
  std::vector<int> stall(n, 0);
  bool any = false;
  for (int i = 0; i < n; ++i) {
    BiScal& q = hs[i];
    std::memset(&q, 0, sizeof(q));
    q.rho = make_double2(rho0[i], rho0[n + i]);
    q.rr = bb[i];
    q.rsd_sq = tol * tol * bb[i];
    q.status = std::isfinite(bb[i]) ? GBC_OK : GBC_ERR_NONFINITE;
    q.active = active[i] && std::isfinite(bb[i]) && bb[i] > q.rsd_sq;
    any |= q.active != 0;
    maxr[i] = at_update[i] = std::sqrt(bb[i]);
  }
  {
    GBC_CUDA(cudaMemcpyAsync(d_sc, hs.data(), sizeof(BiScal) * n, cudaMemcpyHostToDevice, st));
    // the stencil launches of this solve skip right-hand sides whose device flag says converged;
    // the flags are unset, and the iteration graph released, however the solve ends
    static_assert(sizeof(BiScal) % sizeof(int) == 0, "flag stride in ints");
    cudaGraphExec_t exec = nullptr;
    struct SolveScope {
      gbc_ctx* c;
      cudaGraphExec_t& exec;
      ~SolveScope() {
        c->hop_active = nullptr;
        c->hop_active_stride = 0;
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
      }
    } solve_scope{c, exec};
    c->hop_active = &d_sc[0].active;
    c->hop_active_stride = (int)(sizeof(BiScal) / sizeof(int));
    auto body = [&]() {
      if (pa == PREC_DOUBLE) iteration<PrecD, PrecD>(c, po, d_sc, n, x, r, r0, p, v, s, t, te);
      else if (po == PREC_SINGLE) iteration<PrecS, PrecS>(c, po, d_sc, n, x, r, r0, p, v, s, t, te);
      else iteration<PrecS, PrecH>(c, po, d_sc, n, x, r, r0, p, v, s, t, te);
    };
    constexpr int kBlock = 4;
    long long graph_launches = 0;
    int k = 0;
    while (any && k < maxit) {
      const int steps = k == 0 ? 1 : std::min(kBlock, maxit - k);
      if (k > 0 && steps == kBlock && c->use_graphs) {
        if (!exec) {
          cudaGraph_t graph;
          const long long l0 = launch_count();
          GBC_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
          for (int q = 0; q < kBlock; ++q) body();
          GBC_CUDA(cudaStreamEndCapture(st, &graph));
          GBC_CUDA(cudaGraphInstantiate(&exec, graph, 0));
          cudaGraphDestroy(graph);
          graph_launches = launch_count() - l0;
          count_launch(-graph_launches);
        }
        GBC_CUDA(cudaGraphLaunch(exec, st));
        count_launch(graph_launches);
      } else {
        for (int q = 0; q < steps; ++q) body();
      }
      k += steps;
      GBC_CUDA(cudaMemcpyAsync(hs.data(), d_sc, sizeof(BiScal) * n, cudaMemcpyDeviceToHost, st));
      sync(c);
      any = false;
      bool trigger = false;
      for (int i = 0; i < n; ++i) {
        if (!hs[i].active) continue;
        any = true;
        const double rn = std::sqrt(hs[i].rr);
        maxr[i] = std::max(maxr[i], rn);
        if (delta > 0 && rn < delta * maxr[i]) trigger = true;
        if (rn > at_update[i]) trigger = true;  // the recurrence drifted up: check the true residual
      }
      if (any && trigger) {
        // reliable update: r = b - A x with the accumulator-precision operator, rho = (r0, r)
        Spinor ta = sub(workspace(c, S_TA + 20 * pidx(pa), pa, n), 0, n);
        Spinor tea = sub(workspace(c, S_TEA + 20 * pidx(pa), pa, n), 0, n);
        apply_meo(c, pa, false, x, ta, tea, false);
        blas_copy(g, r, b, st);
        for (int i = 0; i < n; ++i) {
          c->h_coef[i] = make_double2(-1.0, 0.0);
          c->h_coef[n + i] = make_double2(1.0, 0.0);
        }
        GBC_CUDA(cudaMemcpyAsync(c->d_ca, c->h_coef, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
        GBC_CUDA(cudaMemcpyAsync(c->d_cb, c->h_coef + n, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
        blas_axpby(g, c->d_ca, ta, c->d_cb, r, st);  // r = b - A x
        blas_norm2(g, r, red(c), st);
        std::vector<double> nr(n);
        GBC_CUDA(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        sync(c);
        std::memcpy(nr.data(), c->h_result, sizeof(double) * n);
        blas_cdot(g, r0, r, red(c), st);
        std::vector<double> rho(2 * n);
        GBC_CUDA(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st));
        sync(c);
        std::memcpy(rho.data(), c->h_result, sizeof(double) * 2 * n);
        for (int i = 0; i < n; ++i) {
          BiScal& q = hs[i];
          if (!q.active) continue;
          q.rr = nr[i];
          q.rho = make_double2(rho[i], rho[n + i]);
          maxr[i] = at_update[i] = std::sqrt(nr[i]);
          // three updates in a row that fail to halve the true residual: the accumulator
          // precision's floor; the FP64 outer loop takes over
          stall[i] = nr[i] > 0.25 * last_nr[i] ? stall[i] + 1 : 0;
          last_nr[i] = nr[i];
          if (!(nr[i] > q.rsd_sq) || stall[i] >= 3 || !std::isfinite(nr[i])) q.active = 0;
        }
        GBC_CUDA(cudaMemcpyAsync(d_sc, hs.data(), sizeof(BiScal) * n, cudaMemcpyHostToDevice, st));
        sync(c);
        ++out.reliable;
      }
    }
    GBC_CUDA(cudaMemcpyAsync(hs.data(), d_sc, sizeof(BiScal) * n, cudaMemcpyDeviceToHost, st));
    sync(c);
  }
  for (int i = 0; i < n; ++i) {
    out.iters[i] = hs[i].iters;
    out.status[i] = hs[i].status != GBC_OK ? hs[i].status : (hs[i].active ? GBC_ERR_NOT_CONVERGED : GBC_OK);
  }
  return out;
}

}  // namespace gbc
