// Explicit instantiation of the hopping kernels for one storage precision (included by
// dslash_{d,s,h}{0,1}.cu with GBC_RECON12 defined).  The launch shapes below are the candidates
// the autotuner chooses from (TX sites x NRB right-hand sides per block, MINB resident blocks).
#pragma once
#include "dslash.cuh"
#include "dslash_async.cuh"
#include "dslash_rpair.cuh"

namespace gbc {

template <typename P, int RECON, int MODE, bool DAG, int REDUCE>
static int hop_shape(const HopArgs& a, HopShape sh, cudaStream_t s) {
  const int nbx = (a.g.Vh + sh.tx - 1) / sh.tx;
  auto go = [&](auto kern, int tx, int nrb) {
    const int ng = (a.nrhs + nrb - 1) / nrb;
    kern<<<(unsigned)(nbx * ng), tx * nrb, 0, s>>>(a);
    return nbx;
  };
#define GBC_SHAPE(TX, NRB, MINB)                                 \
  if (!sh.pair && sh.tx == TX && sh.nrb == NRB && sh.minb == MINB) \
    return go(hop_kernel<P, RECON, MODE, DAG, REDUCE, TX, NRB, MINB>, TX, NRB);
  if constexpr (std::is_same<P, PrecDF>::value) {
    // double-float arithmetic: about ten times the instructions of the FP32 kernel, so only the
    // shapes without a tight register bound
    GBC_SHAPE(128, 1, 1)
    GBC_SHAPE(32, 4, 1)
    GBC_SHAPE(64, 2, 4)
    return -1;
  } else {
    GBC_SHAPE(128, 1, 1)
    GBC_SHAPE(128, 1, 6)
    GBC_SHAPE(32, 4, 1)
    GBC_SHAPE(32, 4, 5)
    GBC_SHAPE(64, 2, 4)
    GBC_SHAPE(32, 12, 2)
  }
#undef GBC_SHAPE
  if constexpr (std::is_same<P, PrecH>::value) {
    if (sh.pair == 3) {
      // two right-hand sides per thread: blocks of TS sites x NRB right-hand sides, TS NRB / 2 threads
      if (a.nrhs & 1) return -1;
#define GBC_RPAIR(TS, NRB, MINB)                                                          \
  if (sh.tx == TS && sh.nrb == NRB && sh.minb == MINB) {                                  \
    const int ng = (a.nrhs + NRB - 1) / NRB;                                              \
    hop_kernel_rp<RECON, MODE, DAG, REDUCE, TS, NRB, MINB><<<(unsigned)(nbx * ng), TS * NRB / 2, 0, s>>>(a); \
    return nbx;                                                                           \
  }
      GBC_RPAIR(32, 12, 2)
      GBC_RPAIR(16, 12, 5)
      GBC_RPAIR(16, 12, 4)
      GBC_RPAIR(16, 4, 10)
#undef GBC_RPAIR
      return -1;
    }
    if (sh.nrb != 1) return -1;
    if (sh.pair == 1) {
      // two sites per thread: blocks of TX threads cover 2 TX sites
      if (a.g.L[3] & 1) return -1;
      auto go2 = [&](auto kern, int tx) {
        const int nbp = (a.g.Vh / 2 + tx - 1) / tx;
        kern<<<(unsigned)(nbp * a.nrhs), tx, 0, s>>>(a);
        return nbp;
      };
#define GBC_PAIR(TX, MINB) \
  if (sh.tx == TX && sh.minb == MINB) return go2(hop_kernel_pair<RECON, MODE, DAG, REDUCE, TX, MINB>, TX);
      GBC_PAIR(128, 2)
      GBC_PAIR(128, 3)
      GBC_PAIR(64, 6)
#undef GBC_PAIR
    } else if (sh.pair == 2) {
      // the next hops' loads in flight through a shared-memory ring (one site per thread)
#define GBC_ASYNC(TX, MINB) \
  if (sh.tx == TX && sh.minb == MINB) return go(hop_kernel_async<RECON, MODE, DAG, REDUCE, TX, MINB>, TX, 1);
      GBC_ASYNC(128, 3)
      GBC_ASYNC(128, 4)
      GBC_ASYNC(64, 8)
#undef GBC_ASYNC
    }
  }
  return -1;
}

template <typename P, int RECON, bool DAG>
static int hop_mode_reduce(int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);

template <typename P, int RECON, bool DAG>
static int hop_mode(int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  if constexpr (std::is_same<P, PrecDF>::value) {
    // the outer residuals and the Schur prep apply the operator without fused reductions
    if (reduce) return -1;
    switch (mode) {
      case HOP_PLAIN: return hop_shape<P, RECON, HOP_PLAIN, DAG, RED_NONE>(a, sh, s);
      case HOP_CLOV: return hop_shape<P, RECON, HOP_CLOV, DAG, RED_NONE>(a, sh, s);
      case HOP_XPAY: return hop_shape<P, RECON, HOP_XPAY, DAG, RED_NONE>(a, sh, s);
    }
    return -1;
  } else {
    return hop_mode_reduce<P, RECON, DAG>(mode, reduce, a, sh, s);
  }
}

template <typename P, int RECON, bool DAG>
static int hop_mode_reduce(int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  switch (mode) {
    case HOP_PLAIN: return reduce ? -1 : hop_shape<P, RECON, HOP_PLAIN, DAG, RED_NONE>(a, sh, s);
    case HOP_CLOV: return reduce ? -1 : hop_shape<P, RECON, HOP_CLOV, DAG, RED_NONE>(a, sh, s);
    case HOP_XPAY:
      if (reduce == RED_NORM) return hop_shape<P, RECON, HOP_XPAY, DAG, RED_NORM>(a, sh, s);
      if (reduce == RED_DOT_SELF) {
        // BiCGStab applies M~ itself, never its dagger: the variant exists for isign = PLUS only
        if constexpr (!DAG) return hop_shape<P, RECON, HOP_XPAY, DAG, RED_DOT_SELF>(a, sh, s);
        return -1;
      }
      if (reduce == RED_DOT_AUX) {
        if constexpr (!DAG) return hop_shape<P, RECON, HOP_XPAY, DAG, RED_DOT_AUX>(a, sh, s);
        return -1;
      }
      return hop_shape<P, RECON, HOP_XPAY, DAG, RED_NONE>(a, sh, s);
  }
  return -1;
}

template <typename P, bool DAG>
static int hop_recon(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  if (recon == 18) return hop_mode<P, 18, DAG>(mode, reduce, a, sh, s);
#if GBC_RECON12
  if (recon == 12) return hop_mode<P, 12, DAG>(mode, reduce, a, sh, s);
#endif
  return -1;
}

// several lattices in one launch (work table of (lattice, site block), 128-site blocks)
template <typename P, int RECON, bool DAG>
static int hop_multi_mode(int mode, int reduce, const HopArgs* args, const int2* work, int nwork, cudaStream_t s) {
  switch (mode) {
    case HOP_PLAIN: hop_kernel_multi<P, RECON, HOP_PLAIN, DAG, RED_NONE><<<nwork, 128, 0, s>>>(args, work); return nwork;
    case HOP_CLOV: hop_kernel_multi<P, RECON, HOP_CLOV, DAG, RED_NONE><<<nwork, 128, 0, s>>>(args, work); return nwork;
    case HOP_XPAY:
      if (reduce == RED_DOT_SELF || reduce == RED_DOT_AUX) return -1;
      if (reduce) hop_kernel_multi<P, RECON, HOP_XPAY, DAG, RED_NORM><<<nwork, 128, 0, s>>>(args, work);
      else hop_kernel_multi<P, RECON, HOP_XPAY, DAG, RED_NONE><<<nwork, 128, 0, s>>>(args, work);
      return nwork;
  }
  return -1;
}

template <typename P, bool DAG>
static int hop_multi_recon(int recon, int mode, int reduce, const HopArgs* args, const int2* work, int nwork,
                           cudaStream_t s) {
  if (recon == 18) return hop_multi_mode<P, 18, DAG>(mode, reduce, args, work, nwork, s);
#if GBC_RECON12
  if (recon == 12) return hop_multi_mode<P, 12, DAG>(mode, reduce, args, work, nwork, s);
#endif
  return -1;
}

}  // namespace gbc
