// Explicit instantiation of the mixed-precision multi-right-hand-side hopping kernel (fp16 storage,
// dslash_mr.cuh) for one isign: the launch shapes of kHopShapes with pair = 4.
#pragma once
#include "dslash_mr.cuh"

namespace gbc {

template <int RECON, int MODE, bool DAG, int REDUCE>
static int hop_shape_mr(const HopArgs& a, HopShape sh, cudaStream_t s) {
#define GBC_MR(TS, NRB, MINB)                                                                         \
  if (sh.tx == TS && sh.nrb == NRB && sh.minb == MINB) {                                               \
    const int nbx = (a.g.Vh + TS - 1) / TS;                                                            \
    const int ng = (a.nrhs + NRB - 1) / NRB;                                                           \
    hop_kernel_mr<RECON, MODE, DAG, REDUCE, TS, NRB, MINB><<<(unsigned)(nbx * ng), TS * NRB, 0, s>>>(a); \
    return nbx;                                                                                        \
  }
  GBC_MR(16, 12, 3)
  GBC_MR(32, 6, 3)
  GBC_MR(32, 12, 2)
  GBC_MR(32, 4, 5)
#undef GBC_MR
  return -1;
}

template <int RECON, bool DAG>
static int hop_mode_mr(int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  switch (mode) {
    case HOP_PLAIN: return reduce ? -1 : hop_shape_mr<RECON, HOP_PLAIN, DAG, RED_NONE>(a, sh, s);
    case HOP_CLOV: return reduce ? -1 : hop_shape_mr<RECON, HOP_CLOV, DAG, RED_NONE>(a, sh, s);
    case HOP_XPAY:
      if (reduce == RED_NORM) return hop_shape_mr<RECON, HOP_XPAY, DAG, RED_NORM>(a, sh, s);
      if (reduce == RED_DOT_SELF) {
        if constexpr (!DAG) return hop_shape_mr<RECON, HOP_XPAY, DAG, RED_DOT_SELF>(a, sh, s);
        return -1;
      }
      return hop_shape_mr<RECON, HOP_XPAY, DAG, RED_NONE>(a, sh, s);
  }
  return -1;
}

template <bool DAG>
static int hop_launch_mr_impl(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  if (sh.pair != 4) return -1;
  if (recon == 18) return hop_mode_mr<18, DAG>(mode, reduce, a, sh, s);
  if (recon == 12) return hop_mode_mr<12, DAG>(mode, reduce, a, sh, s);
  return -1;
}

}  // namespace gbc
