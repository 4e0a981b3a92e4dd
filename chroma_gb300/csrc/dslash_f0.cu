// Hopping kernels on FP64-stored fields in double-float arithmetic, isign = PLUS.
#define GBC_RECON12 0
#include "dslash_inst.cuh"

namespace gbc {
int hop_launch_f0(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  return hop_recon<PrecDF, false>(recon, mode, reduce, a, sh, s);
}
}  // namespace gbc
