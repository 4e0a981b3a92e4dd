// The non-stencil part of one CGNE iteration for every lattice of a batch, each as ONE launch:
// alpha from the stencil's |M~ p|^2 partials, the fused update x += a p, r -= a q with |r|^2
// partials, beta, and p = r + b p.  The site kernels walk the batch's work table of
// (lattice, 128-site block) pairs, like hop_kernel_multi; the scalar kernels run one block per
// lattice and sum that lattice's partials in a fixed order (bitwise repeatable), then apply the
// InvCG2 scalar recursion (invcg2.cc:153-221) to the lattice's CGScalars.
#include "batch_ops.cuh"

namespace gbc {
namespace {

constexpr int kSites = kBatchSites;

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

// e += a p;  r -= a q;  partial |r|^2 per block   (e, r in PA; p, q in PO)
template <typename PA, typename PO>
__global__ void __launch_bounds__(kSites) update_kernel(const LatCg* lat, const int2* work) {
  const int2 w = work[blockIdx.x];
  const LatCg& l = lat[w.x];
  batch_update_block<PA, PO>(l, w.y, l.cg->a);
}

// p = r + b p   (r in PA, p in PO)
template <typename PA, typename PO>
__global__ void __launch_bounds__(kSites) xpay_kernel(const LatCg* lat, const int2* work) {
  const int2 w = work[blockIdx.x];
  const LatCg& l = lat[w.x];
  batch_xpay_block<PA, PO>(l, w.y, l.cg->b);
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
