// Vector updates of one lattice's batched CGNE on one work item (lattice, 128-site block), called
// by a whole 128-thread block.  Shared by the one-launch-per-step kernels (batch_kernels.cu) and the
// persistent kernel (batch_persistent.cuh); the InvCG2 updates of invcg2.cc:165-220.
#pragma once
#include "gbc_device.cuh"

namespace gbc {

constexpr int kBatchSites = 128;  // sites per work-table block (the stencil's block)

template <typename P>
__device__ __forceinline__ void ldf(cplx<typename P::real> (&x)[12], const Spinor& f, int idx) {
  load_spinor<P>(x, f.v, f.norm, idx, f.stride);
}
template <typename P>
__device__ __forceinline__ void stf(const Spinor& f, int idx, const cplx<typename P::real> (&x)[12]) {
  store_spinor<P>(f.v, f.norm, idx, f.stride, x);
}

// e += a p;  r -= a q;  |r|^2 of the block -> l.upd_part[sblock]   (e, r in PA; p, q in PO).
// Site and warp sums in the compute precision, the block sum in FP64, in a fixed order.
template <typename PA, typename PO>
__device__ __forceinline__ void batch_update_block(const LatCg& l, int sblock, double alpha) {
  const int idx = sblock * kBatchSites + threadIdx.x;
  using T = typename PA::real;
  T acc = 0;
  if (idx < l.Vh) {
    cplx<T> es[12], rs[12];
    cplx<typename PO::real> ps[12], qs[12];
    ldf<PA>(es, l.e, idx);
    ldf<PA>(rs, l.r, idx);
    ldf<PO>(ps, l.p, idx);
    ldf<PO>(qs, l.q, idx);
    const T al = (T)alpha;
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
  __shared__ double sh[kBatchSites / 32];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kBatchSites / 32; ++q) s += sh[q];
    l.upd_part[sblock] = s;
  }
  __syncthreads();  // sh is reused by the next call
}

// p = r + b p   (r in PA, p in PO)
template <typename PA, typename PO>
__device__ __forceinline__ void batch_xpay_block(const LatCg& l, int sblock, double beta) {
  const int idx = sblock * kBatchSites + threadIdx.x;
  if (idx >= l.Vh) return;
  using T = typename PO::real;
  cplx<typename PA::real> rs[12];
  cplx<T> ps[12];
  ldf<PA>(rs, l.r, idx);
  ldf<PO>(ps, l.p, idx);
  const T be = (T)beta;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    ps[k].re = fmadd(be, ps[k].re, (T)rs[k].re);
    ps[k].im = fmadd(be, ps[k].im, (T)rs[k].im);
  }
  stf<PO>(l.p, idx, ps);
}

}  // namespace gbc
