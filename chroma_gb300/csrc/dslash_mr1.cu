// Mixed-precision multi-right-hand-side hopping kernels, fp16 storage, isign = MINUS (dagger).
#include "dslash_mr_inst.cuh"

namespace gbc {
int hop_launch_mr1(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  return hop_launch_mr_impl<true>(recon, mode, reduce, a, sh, s);
}
}  // namespace gbc
