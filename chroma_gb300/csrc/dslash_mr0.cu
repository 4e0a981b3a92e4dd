// Mixed-precision multi-right-hand-side hopping kernels, fp16 storage, isign = PLUS.
#include "dslash_mr_inst.cuh"

namespace gbc {
int hop_launch_mr0(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  return hop_launch_mr_impl<false>(recon, mode, reduce, a, sh, s);
}
}  // namespace gbc
