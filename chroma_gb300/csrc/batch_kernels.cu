// The non-stencil part of one CGNE iteration for every lattice of a batch, each as ONE launch:
// alpha from the stencil's |M~ p|^2 partials, the fused update x += a p, r -= a q with |r|^2
// partials, beta, and p = r + b p.  The site kernels walk the batch's work table of
// (lattice, 128-site block) pairs, like hop_kernel_multi; the scalar kernels run one block per
// lattice and sum that lattice's partials in a fixed order (bitwise repeatable), then apply the
// InvCG2 scalar recursion (invcg2.cc:153-221) to the lattice's CGScalars.
#include "gbc_device.cuh"

namespace gbc {
namespace {

constexpr int kSites = 128;  // sites per work-table block (the stencil's block)

__device__ double block_sum(const double* part, int n) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  return sh[0];
}

__global__ void __launch_bounds__(256) alpha_kernel(const LatCg* lat) {
  const LatCg& l = lat[blockIdx.x];
  const double d = block_sum(l.hop_part, l.nblk);
  if (threadIdx.x == 0) {
    CGScalars s = *l.cg;
    s.d = d;
    s.a = (s.active && s.d > 0.0) ? s.c / s.d : 0.0;
    *l.cg = s;
  }
}

__global__ void __launch_bounds__(256) beta_kernel(const LatCg* lat) {
  const LatCg& l = lat[blockIdx.x];
  const double cp = block_sum(l.upd_part, l.nblk);
  if (threadIdx.x == 0) {
    CGScalars s = *l.cg;
    if (s.active) {
      s.cp = cp;
      s.iters += 1;
      if (!(s.cp > s.rsd_sq)) s.active = 0;
      s.b = (s.active && s.c > 0.0) ? s.cp / s.c : 0.0;
      s.c_prev = s.c;
      s.c = s.cp;
    } else {
      s.b = 0.0;
    }
    *l.cg = s;
  }
}

template <typename P>
__device__ __forceinline__ void ldf(cplx<typename P::real> (&x)[12], const Spinor& f, int idx) {
  load_spinor<P>(x, f.v, f.norm, idx, f.stride);
}
template <typename P>
__device__ __forceinline__ void stf(const Spinor& f, int idx, const cplx<typename P::real> (&x)[12]) {
  store_spinor<P>(f.v, f.norm, idx, f.stride, x);
}

// e += a p;  r -= a q;  partial |r|^2 per block   (e, r in PA; p, q in PO)
template <typename PA, typename PO>
__global__ void __launch_bounds__(kSites) update_kernel(const LatCg* lat, const int2* work) {
  const int2 w = work[blockIdx.x];
  const LatCg& l = lat[w.x];
  const int idx = w.y * kSites + threadIdx.x;
  using T = typename PA::real;
  T acc = 0;  // site and warp sums in the compute precision, block sums in FP64
  if (idx < l.Vh) {
    cplx<T> es[12], rs[12];
    cplx<typename PO::real> ps[12], qs[12];
    ldf<PA>(es, l.e, idx);
    ldf<PA>(rs, l.r, idx);
    ldf<PO>(ps, l.p, idx);
    ldf<PO>(qs, l.q, idx);
    const T al = (T)l.cg->a;
    T s = 0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      es[k].re = fmadd(al, (T)ps[k].re, es[k].re);
      es[k].im = fmadd(al, (T)ps[k].im, es[k].im);
      rs[k].re = fmadd(-al, (T)qs[k].re, rs[k].re);
      rs[k].im = fmadd(-al, (T)qs[k].im, rs[k].im);
      s = fmadd(rs[k].re, rs[k].re, fmadd(rs[k].im, rs[k].im, s));
    }
    stf<PA>(l.e, idx, es);
    stf<PA>(l.r, idx, rs);
    acc = s;
  }
  __shared__ double sh[kSites / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kSites / 32; ++q) s += sh[q];
    l.upd_part[w.y] = s;
  }
}

// p = r + b p   (r in PA, p in PO)
template <typename PA, typename PO>
__global__ void __launch_bounds__(kSites) xpay_kernel(const LatCg* lat, const int2* work) {
  const int2 w = work[blockIdx.x];
  const LatCg& l = lat[w.x];
  const int idx = w.y * kSites + threadIdx.x;
  if (idx >= l.Vh) return;
  using T = typename PO::real;
  cplx<typename PA::real> rs[12];
  cplx<T> ps[12];
  ldf<PA>(rs, l.r, idx);
  ldf<PO>(ps, l.p, idx);
  const T be = (T)l.cg->b;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    ps[k].re = fmadd(be, ps[k].re, (T)rs[k].re);
    ps[k].im = fmadd(be, ps[k].im, (T)rs[k].im);
  }
  stf<PO>(l.p, idx, ps);
}

}  // namespace

// the precision pairs a batch uses: (FP64, FP64) for an FP64 sloppy operator, else FP32
// accumulators with an FP32 or FP16 stencil
#define GBC_PAIR_LAUNCH(KERNEL)                                                  \
  if (pa == PREC_DOUBLE) KERNEL<PrecD, PrecD><<<nwork, kSites, 0, s>>>(lat, work); \
  else if (po == PREC_SINGLE) KERNEL<PrecS, PrecS><<<nwork, kSites, 0, s>>>(lat, work); \
  else KERNEL<PrecS, PrecH><<<nwork, kSites, 0, s>>>(lat, work);                   \
  count_launch();

void batch_cg_alpha(const LatCg* lat, int n, cudaStream_t s) {
  alpha_kernel<<<n, 256, 0, s>>>(lat);
  count_launch();
}
void batch_cg_beta(const LatCg* lat, int n, cudaStream_t s) {
  beta_kernel<<<n, 256, 0, s>>>(lat);
  count_launch();
}
void batch_cg_update(int pa, int po, const LatCg* lat, const int2* work, int nwork, cudaStream_t s) {
  GBC_PAIR_LAUNCH(update_kernel)
}
void batch_xpay(int pa, int po, const LatCg* lat, const int2* work, int nwork, cudaStream_t s) {
  GBC_PAIR_LAUNCH(xpay_kernel)
}
#undef GBC_PAIR_LAUNCH

}  // namespace gbc
