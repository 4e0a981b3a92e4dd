// Dispatch of the double-float hopping kernels on isign.
#include "gbc_kernels.h"

namespace gbc {
int hop_launch_f0(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);
int hop_launch_f1(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);
int hop_launch_df(int recon, int mode, bool dag, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  return dag ? hop_launch_f1(recon, mode, reduce, a, sh, s) : hop_launch_f0(recon, mode, reduce, a, sh, s);
}
}  // namespace gbc
