// Block-vector BLAS for the flexible GMRES: k inner products <V_i, w> in one launch, the
// combination w += sign * sum_i c_i V_i in one launch, and y = a x.  FP64 accumulation,
// per-right-hand-side complex coefficients (FlexibleArnoldiT, syssolver_linop_fgmres_dr.cc:77-195,
// done here as classical Gram-Schmidt applied twice instead of modified Gram-Schmidt).
#include "gbc_device.cuh"
#include "krylov.h"

namespace gbc {
namespace {

constexpr int KT = 256;

template <typename PV, typename PW>
__global__ void __launch_bounds__(KT) multi_cdot_kernel(int Vh, VecList vl, Spinor w, double* partials, int part_stride,
                                                       int nrhs) {
  const int r = blockIdx.y;
  const int i = blockIdx.z;
  const Spinor& v = vl.v[i];
  // thread and warp sums in the compute precision, block sums in FP64 (FP64 per site is slow here)
  using T = typename std::conditional<std::is_same<PV, PrecD>::value || std::is_same<PW, PrecD>::value, double,
                                      float>::type;
  T re = 0, im = 0;
  for (int idx = blockIdx.x * KT + threadIdx.x; idx < Vh; idx += gridDim.x * KT) {
    cplx<typename PV::real> a[12];
    cplx<typename PW::real> b[12];
    load_spinor<PV>(a, (const char*)v.v + (size_t)r * v.rhs_bytes, v.norm ? v.norm + (size_t)r * v.norm_rhs_stride : nullptr,
                    idx, v.stride);
    load_spinor<PW>(b, (const char*)w.v + (size_t)r * w.rhs_bytes, w.norm ? w.norm + (size_t)r * w.norm_rhs_stride : nullptr,
                    idx, w.stride);
    T sr = 0, si = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      sr = fmadd((T)a[k].re, (T)b[k].re, fmadd((T)a[k].im, (T)b[k].im, sr));
      si = fmadd((T)a[k].re, (T)b[k].im, fmadd(-(T)a[k].im, (T)b[k].re, si));
    }
    re += sr;
    im += si;
  }
  __shared__ double sh[2][KT / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    re += __shfl_down_sync(0xffffffffu, re, off);
    im += __shfl_down_sync(0xffffffffu, im, off);
  }
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = (double)re;
    sh[1][threadIdx.x >> 5] = (double)im;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < KT / 32; ++q) s += sh[threadIdx.x][q];
    // row (i, re/im, rhs)
    partials[(((size_t)i * 2 + threadIdx.x) * nrhs + r) * part_stride + blockIdx.x] = s;
  }
}

// w += sign * sum_i coef[i][r] * V_i
template <typename PV, typename PW>
__global__ void __launch_bounds__(KT) multi_caxpy_kernel(int Vh, VecList vl, int k, const double2* coef, Spinor w,
                                                        double sign) {
  const int r = blockIdx.y;
  const int nrhs = gridDim.y;
  using T = typename PW::real;
  for (int idx = blockIdx.x * KT + threadIdx.x; idx < Vh; idx += gridDim.x * KT) {
    cplx<T> acc[12];
    load_spinor<PW>(acc, (const char*)w.v + (size_t)r * w.rhs_bytes, w.norm ? w.norm + (size_t)r * w.norm_rhs_stride : nullptr,
                    idx, w.stride);
    for (int i = 0; i < k; ++i) {
      const Spinor& v = vl.v[i];
      cplx<typename PV::real> a[12];
      load_spinor<PV>(a, (const char*)v.v + (size_t)r * v.rhs_bytes, v.norm ? v.norm + (size_t)r * v.norm_rhs_stride : nullptr,
                      idx, v.stride);
      const double2 cc = coef[(size_t)i * nrhs + r];
      const cplx<T> c{(T)(sign * cc.x), (T)(sign * cc.y)};
#pragma unroll
      for (int q = 0; q < 12; ++q) cmac(acc[q], c, cplx<T>{(T)a[q].re, (T)a[q].im});
    }
    store_spinor<PW>((char*)w.v + (size_t)r * w.rhs_bytes, w.norm ? w.norm + (size_t)r * w.norm_rhs_stride : nullptr, idx,
                     w.stride, acc);
  }
}

// y = a x (y is not read)
template <typename PY, typename PX>
__global__ void __launch_bounds__(KT) cax_kernel(int Vh, const double2* a, Spinor x, Spinor y) {
  const int r = blockIdx.y;
  using T = typename PY::real;
  const double2 ca = a[r];
  const cplx<T> A{(T)ca.x, (T)ca.y};
  for (int idx = blockIdx.x * KT + threadIdx.x; idx < Vh; idx += gridDim.x * KT) {
    cplx<typename PX::real> xs[12];
    load_spinor<PX>(xs, (const char*)x.v + (size_t)r * x.rhs_bytes, x.norm ? x.norm + (size_t)r * x.norm_rhs_stride : nullptr,
                    idx, x.stride);
    cplx<T> ys[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) ys[q] = A * cplx<T>{(T)xs[q].re, (T)xs[q].im};
    store_spinor<PY>((char*)y.v + (size_t)r * y.rhs_bytes, y.norm ? y.norm + (size_t)r * y.norm_rhs_stride : nullptr, idx,
                     y.stride, ys);
  }
}

}  // namespace

#define GBC_K_DISPATCH2(pa, pb, CALL)                                                          \
  do {                                                                                        \
    if (pa == PREC_DOUBLE && pb == PREC_DOUBLE) { using PA = PrecD; using PB = PrecD; CALL; }  \
    else if (pa == PREC_SINGLE && pb == PREC_SINGLE) { using PA = PrecS; using PB = PrecS; CALL; } \
    else if (pa == PREC_SINGLE && pb == PREC_HALF) { using PA = PrecS; using PB = PrecH; CALL; } \
    else if (pa == PREC_HALF && pb == PREC_SINGLE) { using PA = PrecH; using PB = PrecS; CALL; } \
    else if (pa == PREC_HALF && pb == PREC_HALF) { using PA = PrecH; using PB = PrecH; CALL; }  \
    else if (pa == PREC_DOUBLE && pb == PREC_SINGLE) { using PA = PrecD; using PB = PrecS; CALL; } \
    else { using PA = PrecS; using PB = PrecD; CALL; }                                         \
  } while (0)

void multi_cdot(const Geom& g, const VecList& vl, int k, const Spinor& w, const Red& red, cudaStream_t s) {
  dim3 grid(blas_blocks(g), w.nrhs, k);
  GBC_K_DISPATCH2(vl.v[0].prec, w.prec,
                  (multi_cdot_kernel<PA, PB><<<grid, KT, 0, s>>>(g.Vh, vl, w, red.partials, red.part_stride, w.nrhs)));
  count_launch();
  reduce_finalize(red, 2 * k, w.nrhs, grid.x, s);
}

void multi_caxpy(const Geom& g, const VecList& vl, int k, const double2* coef, const Spinor& w, double sign,
                 cudaStream_t s) {
  dim3 grid(blas_blocks(g), w.nrhs);
  GBC_K_DISPATCH2(vl.v[0].prec, w.prec,
                  (multi_caxpy_kernel<PA, PB><<<grid, KT, 0, s>>>(g.Vh, vl, k, coef, w, sign)));
  count_launch();
}

void blas_cax(const Geom& g, const double2* a, const Spinor& x, const Spinor& y, cudaStream_t s) {
  dim3 grid(blas_blocks(g), y.nrhs);
  GBC_K_DISPATCH2(y.prec, x.prec, (cax_kernel<PA, PB><<<grid, KT, 0, s>>>(g.Vh, a, x, y)));
  count_launch();
}

}  // namespace gbc
