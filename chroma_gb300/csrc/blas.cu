// BLAS-1 on checkerboard spinor fields (any storage precision per operand).  Reductions sum a
// thread's sites and a warp's lanes in the operands' compute precision (FP32 unless an operand is
// FP64: GB300's FP64 pipe made per-site FP64 sums the bottleneck of bandwidth-bound kernels), then
// per-warp and per-block sums in FP64 in a fixed grid, then one deterministic finalize pass.  Also the device-side CG scalar logic, so that an iteration
// needs no host round trip (InvCG2, lib/actions/ferm/invert/invcg2.cc:153-221).
#include <string>

#include "gbc_device.cuh"

namespace gbc {

namespace {

constexpr int BLAS_THREADS = 256;

// grid-stride driver: f(idx, rhs, acc) per site; NRED doubles reduced per right-hand side
template <int NRED, class F>
__global__ void __launch_bounds__(BLAS_THREADS) site_kernel(int Vh, F f, double* partials, int part_stride, int nrhs) {
  using A = typename AccOf<F>::type;
  const int r = blockIdx.y;
  A acc[NRED > 0 ? NRED : 1];
#pragma unroll
  for (int q = 0; q < (NRED > 0 ? NRED : 1); ++q) acc[q] = 0;
  for (int idx = blockIdx.x * BLAS_THREADS + threadIdx.x; idx < Vh; idx += gridDim.x * BLAS_THREADS) f(idx, r, acc);
  if constexpr (NRED > 0) {
    __shared__ double sh[NRED][BLAS_THREADS / 32];
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
      for (int w = 0; w < BLAS_THREADS / 32; ++w) s += sh[threadIdx.x][w];
      partials[((size_t)threadIdx.x * nrhs + r) * part_stride + blockIdx.x] = s;
    }
  }
}

template <typename P>
__device__ __forceinline__ void ld(cplx<typename P::real> (&x)[12], const Spinor& f, int idx, int r) {
  load_spinor<P>(x, (const char*)f.v + (size_t)r * f.rhs_bytes, f.norm ? f.norm + (size_t)r * f.norm_rhs_stride : nullptr,
                 idx, f.stride);
}
template <typename P>
__device__ __forceinline__ void st(const Spinor& f, int idx, int r, const cplx<typename P::real> (&x)[12]) {
  store_spinor<P>((char*)f.v + (size_t)r * f.rhs_bytes, f.norm ? f.norm + (size_t)r * f.norm_rhs_stride : nullptr, idx,
                  f.stride, x);
}

template <typename PY, typename PX>
struct CopyF {
  Spinor y, x;
  __device__ void operator()(int idx, int r, double*) const {
    cplx<typename PX::real> a[12];
    ld<PX>(a, x, idx, r);
    cplx<typename PY::real> b[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) b[k] = {(typename PY::real)a[k].re, (typename PY::real)a[k].im};
    st<PY>(y, idx, r, b);
  }
};

template <typename P>
struct ZeroF {
  Spinor y;
  __device__ void operator()(int idx, int r, double*) const {
    cplx<typename P::real> b[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) b[k] = {0, 0};
    st<P>(y, idx, r, b);
  }
};

template <typename P>
struct Norm2F {
  using Acc = typename P::real;  // site and thread sums in the field's compute precision
  Spinor x;
  __device__ void operator()(int idx, int r, Acc* acc) const {
    cplx<typename P::real> a[12];
    ld<P>(a, x, idx, r);
    using T = typename P::real;
    T s = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) s = fmadd(a[k].re, a[k].re, fmadd(a[k].im, a[k].im, s));
    acc[0] += s;
  }
};

template <typename PX, typename PY>
struct CdotF {
  using Acc = typename std::conditional<std::is_same<PX, PrecD>::value || std::is_same<PY, PrecD>::value, double,
                                        float>::type;
  Spinor x, y;
  __device__ void operator()(int idx, int r, Acc* acc) const {
    cplx<typename PX::real> a[12];
    cplx<typename PY::real> b[12];
    ld<PX>(a, x, idx, r);
    ld<PY>(b, y, idx, r);
    using T = Acc;
    T re = 0, im = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      re = fmadd((T)a[k].re, (T)b[k].re, fmadd((T)a[k].im, (T)b[k].im, re));
      im = fmadd((T)a[k].re, (T)b[k].im, fmadd(-(T)a[k].im, (T)b[k].re, im));
    }
    acc[0] += re;
    acc[1] += im;
  }
};

// y = a x + b y, complex a, b per right-hand side (FGMRES)
template <typename PY, typename PX>
struct AxpbyF {
  const double2* a;
  const double2* b;
  Spinor x, y;
  __device__ void operator()(int idx, int r, double*) const {
    using T = typename PY::real;
    cplx<typename PX::real> xs[12];
    cplx<T> ys[12];
    ld<PX>(xs, x, idx, r);
    ld<PY>(ys, y, idx, r);
    const double2 ca = a[r], cb = b[r];
    const cplx<T> A{(T)ca.x, (T)ca.y}, B{(T)cb.x, (T)cb.y};
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      cplx<T> xv{(T)xs[k].re, (T)xs[k].im};
      ys[k] = A * xv + B * ys[k];
    }
    st<PY>(y, idx, r, ys);
  }
};

// x += a p; r -= a q; acc = |r|^2   (x, r in PA;  p, q in PO)
template <typename PA, typename PO>
struct CgUpdateF {
  using Acc = typename PA::real;
  const double* a;
  Spinor x, p, r, q;
  __device__ void operator()(int idx, int rr, Acc* acc) const {
    using T = typename PA::real;
    cplx<T> xs[12], rs[12];
    cplx<typename PO::real> ps[12], qs[12];
    ld<PA>(xs, x, idx, rr);
    ld<PA>(rs, r, idx, rr);
    ld<PO>(ps, p, idx, rr);
    ld<PO>(qs, q, idx, rr);
    const T al = (T)a[rr];
    T s = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      xs[k].re = fmadd(al, (T)ps[k].re, xs[k].re);
      xs[k].im = fmadd(al, (T)ps[k].im, xs[k].im);
      rs[k].re = fmadd(-al, (T)qs[k].re, rs[k].re);
      rs[k].im = fmadd(-al, (T)qs[k].im, rs[k].im);
      s = fmadd(rs[k].re, rs[k].re, fmadd(rs[k].im, rs[k].im, s));
    }
    st<PA>(x, idx, rr, xs);
    st<PA>(r, idx, rr, rs);
    acc[0] += s;
  }
};

// p = r + b p    (r in PA, p in PO)
template <typename PA, typename PO>
struct XpayF {
  const double* b;
  Spinor r, p;
  __device__ void operator()(int idx, int rr, double*) const {
    using T = typename PO::real;
    cplx<typename PA::real> rs[12];
    cplx<T> ps[12];
    ld<PA>(rs, r, idx, rr);
    ld<PO>(ps, p, idx, rr);
    const T be = (T)b[rr];
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      ps[k].re = fmadd(be, ps[k].re, (T)rs[k].re);
      ps[k].im = fmadd(be, ps[k].im, (T)rs[k].im);
    }
    st<PO>(p, idx, rr, ps);
  }
};

// y = x - y; acc = |y|^2
template <typename P>
struct XmyNormF {
  using Acc = typename P::real;
  Spinor x, y;
  __device__ void operator()(int idx, int r, Acc* acc) const {
    cplx<typename P::real> xs[12], ys[12];
    ld<P>(xs, x, idx, r);
    ld<P>(ys, y, idx, r);
    typename P::real s = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      ys[k] = xs[k] - ys[k];
      s = fmadd(ys[k].re, ys[k].re, fmadd(ys[k].im, ys[k].im, s));
    }
    st<P>(y, idx, r, ys);
    acc[0] += s;
  }
};

// y = x - y + tw i gamma_5 x;  acc = |y|^2   (the last step of the symmetric operator with a
// twisted-mass term; gamma_5 = diag(1, 1, -1, -1) in the DeGrand-Rossi basis)
template <typename P>
struct XmyTwistNormF {
  using Acc = typename P::real;
  Spinor x, y;
  double tw;
  __device__ void operator()(int idx, int r, Acc* acc) const {
    using T = typename P::real;
    cplx<T> xs[12], ys[12];
    ld<P>(xs, x, idx, r);
    ld<P>(ys, y, idx, r);
    T s = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      const T t5 = (T)(k < 6 ? tw : -tw);
      ys[k] = xs[k] - ys[k] + t5 * timesI(xs[k]);
      s = fmadd(ys[k].re, ys[k].re, fmadd(ys[k].im, ys[k].im, s));
    }
    st<P>(y, idx, r, ys);
    acc[0] += s;
  }
};

// y += sigma_r x;  acc = Re <x, y>   (the shifted normal operator of the multi-shift refinement:
// y = M~^dag M~ x on entry, (M~^dag M~ + sigma) x and x^dag (M~^dag M~ + sigma) x on exit)
template <typename P>
struct ShiftDotF {
  using Acc = typename P::real;
  const double* sigma;
  Spinor x, y;
  __device__ void operator()(int idx, int r, Acc* acc) const {
    using T = typename P::real;
    cplx<T> xs[12], ys[12];
    ld<P>(xs, x, idx, r);
    ld<P>(ys, y, idx, r);
    const T sg = (T)sigma[r];
    T d = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      ys[k].re = fmadd(sg, xs[k].re, ys[k].re);
      ys[k].im = fmadd(sg, xs[k].im, ys[k].im);
      d = fmadd(xs[k].re, ys[k].re, fmadd(xs[k].im, ys[k].im, d));
    }
    st<P>(y, idx, r, ys);
    acc[0] += d;
  }
};

// y += sigma_r x
template <typename P>
struct ShiftAxpyF {
  const double* sigma;
  Spinor x, y;
  __device__ void operator()(int idx, int r, double*) const {
    using T = typename P::real;
    cplx<T> xs[12], ys[12];
    ld<P>(xs, x, idx, r);
    ld<P>(ys, y, idx, r);
    const T sg = (T)sigma[r];
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      ys[k].re = fmadd(sg, xs[k].re, ys[k].re);
      ys[k].im = fmadd(sg, xs[k].im, ys[k].im);
    }
    st<P>(y, idx, r, ys);
  }
};

// x += y  (x in PX, y in PY)
template <typename PX, typename PY>
struct XpyF {
  Spinor x, y;
  __device__ void operator()(int idx, int r, double*) const {
    using T = typename PX::real;
    cplx<T> xs[12];
    cplx<typename PY::real> ys[12];
    ld<PX>(xs, x, idx, r);
    ld<PY>(ys, y, idx, r);
#pragma unroll
    for (int k = 0; k < 12; ++k) xs[k] = xs[k] + cplx<T>{(T)ys[k].re, (T)ys[k].im};
    st<PX>(x, idx, r, xs);
  }
};

// x -= y (y may be lower precision);  acc = |x|^2
template <typename PX, typename PY>
struct XsubNormF {
  using Acc = typename PX::real;
  Spinor x, y;
  __device__ void operator()(int idx, int r, Acc* acc) const {
    using T = typename PX::real;
    cplx<T> xs[12];
    cplx<typename PY::real> ys[12];
    ld<PX>(xs, x, idx, r);
    ld<PY>(ys, y, idx, r);
    T s = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      xs[k] = xs[k] - cplx<T>{(T)ys[k].re, (T)ys[k].im};
      s = fmadd(xs[k].re, xs[k].re, fmadd(xs[k].im, xs[k].im, s));
    }
    st<PX>(x, idx, r, xs);
    acc[0] += s;
  }
};

__global__ void finalize_kernel(const double* partials, int part_stride, int nblocks, double* result) {
  // one block per (quantity, rhs); fixed-order tree => bitwise repeatable
  const int qr = blockIdx.x;
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += 256) s += partials[(size_t)qr * part_stride + i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) result[qr] = sh[0];
}

__global__ void cg_alpha_kernel(CGScalars* st, const double* red_d, double* a_out, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  CGScalars s = st[r];
  s.d = red_d[r];
  s.a = (s.active && s.d > 0.0) ? s.c / s.d : 0.0;
  a_out[r] = s.a;
  st[r] = s;
}

__global__ void cg_beta_kernel(CGScalars* st, const double* red_r, double* b_out, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  CGScalars s = st[r];
  if (s.active) {
    s.cp = red_r[r];
    s.iters += 1;
    if (!(s.cp > s.rsd_sq)) s.active = 0;  // converged (or non-finite: stops and is reported)
    s.b = (s.active && s.c > 0.0) ? s.cp / s.c : 0.0;
    s.c_prev = s.c;
    s.c = s.cp;
  } else {
    s.b = 0.0;
  }
  b_out[r] = s.b;
  st[r] = s;
}

template <int NRED, class F>
void run(const Geom& g, int nrhs, const F& f, const Red* red, cudaStream_t s) {
  dim3 grid(blas_blocks(g), nrhs);
  site_kernel<NRED, F><<<grid, BLAS_THREADS, 0, s>>>(g.Vh, f, red ? red->partials : nullptr,
                                                     red ? red->part_stride : 0, nrhs);
  count_launch();
  if (NRED > 0) reduce_finalize(*red, NRED, nrhs, grid.x, s);
}

}  // namespace

int blas_blocks(const Geom& g) {
  // a multiple of the 152 SMs that keeps every block busy
  int want = (g.Vh + BLAS_THREADS - 1) / BLAS_THREADS;
  int cap = 152 * 8;
  return want < cap ? want : cap;
}

void reduce_finalize(const Red& red, int nred, int nrhs, int nblocks, cudaStream_t s) {
  finalize_kernel<<<nred * nrhs, 256, 0, s>>>(red.partials, red.part_stride, nblocks, red.result);
  count_launch();
}

#define GBC_DISPATCH1(prec, CALL) \
  switch (prec) {                 \
    case PREC_DOUBLE: { using PA = PrecD; CALL; } break; \
    case PREC_SINGLE: { using PA = PrecS; CALL; } break; \
    default: { using PA = PrecH; CALL; } break;          \
  }
#define GBC_DISPATCH2(pa, pb, CALL)                                    \
  switch (pa) {                                                        \
    case PREC_DOUBLE: { using PA = PrecD;                              \
      switch (pb) { case PREC_DOUBLE: { using PB = PrecD; CALL; } break; \
                    case PREC_SINGLE: { using PB = PrecS; CALL; } break; \
                    default: { using PB = PrecH; CALL; } } } break;      \
    case PREC_SINGLE: { using PA = PrecS;                              \
      switch (pb) { case PREC_DOUBLE: { using PB = PrecD; CALL; } break; \
                    case PREC_SINGLE: { using PB = PrecS; CALL; } break; \
                    default: { using PB = PrecH; CALL; } } } break;      \
    default: { using PA = PrecH;                                       \
      switch (pb) { case PREC_DOUBLE: { using PB = PrecD; CALL; } break; \
                    case PREC_SINGLE: { using PB = PrecS; CALL; } break; \
                    default: { using PB = PrecH; CALL; } } } break;      \
  }

void blas_copy(const Geom& g, const Spinor& y, const Spinor& x, cudaStream_t s) {
  GBC_DISPATCH2(y.prec, x.prec, (run<0>(g, y.nrhs, CopyF<PA, PB>{y, x}, nullptr, s)));
}
void blas_zero(const Geom& g, const Spinor& y, cudaStream_t s) {
  GBC_DISPATCH1(y.prec, (run<0>(g, y.nrhs, ZeroF<PA>{y}, nullptr, s)));
}
void blas_axpby(const Geom& g, const double2* a, const Spinor& x, const double2* b, const Spinor& y, cudaStream_t s) {
  GBC_DISPATCH2(y.prec, x.prec, (run<0>(g, y.nrhs, AxpbyF<PA, PB>{a, b, x, y}, nullptr, s)));
}
void blas_norm2(const Geom& g, const Spinor& x, const Red& r, cudaStream_t s) {
  GBC_DISPATCH1(x.prec, (run<1>(g, x.nrhs, Norm2F<PA>{x}, &r, s)));
}
void blas_cdot(const Geom& g, const Spinor& x, const Spinor& y, const Red& r, cudaStream_t s) {
  GBC_DISPATCH2(x.prec, y.prec, (run<2>(g, x.nrhs, CdotF<PA, PB>{x, y}, &r, s)));
}
void blas_cg_update(const Geom& g, const double* a, const Spinor& x, const Spinor& p, const Spinor& r, const Spinor& q,
                    const Red& red, cudaStream_t s) {
  GBC_DISPATCH2(x.prec, p.prec, (run<1>(g, x.nrhs, CgUpdateF<PA, PB>{a, x, p, r, q}, &red, s)));
}
void blas_xpay(const Geom& g, const Spinor& r, const double* b, const Spinor& p, cudaStream_t s) {
  GBC_DISPATCH2(r.prec, p.prec, (run<0>(g, r.nrhs, XpayF<PA, PB>{b, r, p}, nullptr, s)));
}
void blas_xmy_norm2(const Geom& g, const Spinor& x, const Spinor& y, const Red& red, cudaStream_t s) {
  GBC_DISPATCH1(x.prec, (run<1>(g, x.nrhs, XmyNormF<PA>{x, y}, &red, s)));
}
void blas_xmy_twist_norm2(const Geom& g, const Spinor& x, const Spinor& y, double tw, const Red& red,
                          cudaStream_t s) {
  GBC_DISPATCH1(x.prec, (run<1>(g, x.nrhs, XmyTwistNormF<PA>{x, y, tw}, &red, s)));
}
void blas_shift_dot(const Geom& g, const double* sigma, const Spinor& x, const Spinor& y, const Red& red,
                    cudaStream_t s) {
  GBC_DISPATCH1(x.prec, (run<1>(g, x.nrhs, ShiftDotF<PA>{sigma, x, y}, &red, s)));
}
void blas_shift_axpy(const Geom& g, const double* sigma, const Spinor& x, const Spinor& y, cudaStream_t s) {
  GBC_DISPATCH1(x.prec, (run<0>(g, x.nrhs, ShiftAxpyF<PA>{sigma, x, y}, nullptr, s)));
}
void blas_xpy(const Geom& g, const Spinor& x, const Spinor& y, cudaStream_t s) {
  GBC_DISPATCH2(x.prec, y.prec, (run<0>(g, x.nrhs, XpyF<PA, PB>{x, y}, nullptr, s)));
}
void blas_xsub_norm2(const Geom& g, const Spinor& x, const Spinor& y, const Red& red, cudaStream_t s) {
  GBC_DISPATCH2(x.prec, y.prec, (run<1>(g, x.nrhs, XsubNormF<PA, PB>{x, y}, &red, s)));
}

void cg_alpha(CGScalars* st, const double* red_d, double* a_out, int nrhs, cudaStream_t s) {
  cg_alpha_kernel<<<1, 32, 0, s>>>(st, red_d, a_out, nrhs);
  count_launch();
}
void cg_beta(CGScalars* st, const double* red_r, double* b_out, int nrhs, cudaStream_t s) {
  cg_beta_kernel<<<1, 32, 0, s>>>(st, red_r, b_out, nrhs);
  count_launch();
}

}  // namespace gbc

namespace gbc {
namespace {
template <typename P>
struct CloverF {
  const void* clov;
  Spinor out, in;
  int stride;
  __device__ void operator()(int idx, int r, double*) const {
    using T = typename P::real;
    cplx<T> x[12], y[12];
    ld<P>(x, in, idx, r);
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      T d[6];
      cplx<T> o[15], xb[6], yb[6];
      load_clover_block<P>(d, o, clov, idx, stride, b);
#pragma unroll
      for (int k = 0; k < 6; ++k) xb[k] = x[6 * b + k];
      clover_block_mul(yb, d, o, xb);
#pragma unroll
      for (int k = 0; k < 6; ++k) y[6 * b + k] = yb[k];
    }
    st<P>(out, idx, r, y);
  }
};
}  // namespace

void blas_clover(const Geom& g, const void* clov, const Spinor& out, const Spinor& in, cudaStream_t s, bool df) {
  if (df) {
    if (in.prec != PREC_DOUBLE || out.prec != PREC_DOUBLE) throw std::string("double-float clover needs FP64 fields");
    run<0>(g, in.nrhs, CloverF<PrecDF>{clov, out, in, g.stride}, nullptr, s);
    return;
  }
  GBC_DISPATCH1(in.prec, (run<0>(g, in.nrhs, CloverF<PA>{clov, out, in, g.stride}, nullptr, s)));
}

namespace {
__global__ void split_kernel(const double* in, float2* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const df64 v = df64_from_bits(in[i]);
    out[i] = make_float2(v.hi, v.lo);
  }
}
}  // namespace

void split_df64(const double* in, float2* out, size_t n, cudaStream_t s) {
  split_kernel<<<1216, 256, 0, s>>>(in, out, n);
  count_launch();
}
}  // namespace gbc
