// Hopping kernels on FP64-stored fields in double-float arithmetic, isign = MINUS.
#define GBC_RECON12 0
#include "dslash_inst.cuh"

namespace gbc {
int hop_launch_f1(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  return hop_recon<PrecDF, true>(recon, mode, reduce, a, sh, s);
}
}  // namespace gbc
