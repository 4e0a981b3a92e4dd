// Explicit instantiation of the hopping kernels for one storage precision (included by
// dslash_{d,s,h}.cu with GBC_PREC, GBC_LAUNCH_NAME and GBC_RECONS defined).
#pragma once
#include "dslash.cuh"

namespace gbc {

template <typename P, int RECON, int MODE, bool DAG, bool REDUCE>
static int hop_shape(const HopArgs& a, HopShape sh, cudaStream_t s) {
  const int nbx = (a.g.Vh + sh.tx - 1) / sh.tx;
  auto go = [&](auto kern, int tx, int nrb) {
    dim3 grid(nbx, (a.nrhs + nrb - 1) / nrb);
    kern<<<grid, tx * nrb, 0, s>>>(a);
    return nbx;
  };
  if (sh.tx == 128 && sh.nrb == 1) return go(hop_kernel<P, RECON, MODE, DAG, REDUCE, 128, 1>, 128, 1);
  if (sh.tx == 64 && sh.nrb == 1) return go(hop_kernel<P, RECON, MODE, DAG, REDUCE, 64, 1>, 64, 1);
  if (sh.tx == 32 && sh.nrb == 4) return go(hop_kernel<P, RECON, MODE, DAG, REDUCE, 32, 4>, 32, 4);
  if (sh.tx == 32 && sh.nrb == 12) return go(hop_kernel<P, RECON, MODE, DAG, REDUCE, 32, 12>, 32, 12);
  return -1;
}

template <typename P, int RECON, bool DAG>
static int hop_mode(int mode, bool reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  switch (mode) {
    case HOP_PLAIN: return hop_shape<P, RECON, HOP_PLAIN, DAG, false>(a, sh, s);
    case HOP_CLOV: return hop_shape<P, RECON, HOP_CLOV, DAG, false>(a, sh, s);
    case HOP_XPAY:
      return reduce ? hop_shape<P, RECON, HOP_XPAY, DAG, true>(a, sh, s)
                    : hop_shape<P, RECON, HOP_XPAY, DAG, false>(a, sh, s);
  }
  return -1;
}

template <typename P, bool DAG>
static int hop_recon(int recon, int mode, bool reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  if (recon == 18) return hop_mode<P, 18, DAG>(mode, reduce, a, sh, s);
#if GBC_RECON12
  if (recon == 12) return hop_mode<P, 12, DAG>(mode, reduce, a, sh, s);
#endif
  return -1;
}

}  // namespace gbc
