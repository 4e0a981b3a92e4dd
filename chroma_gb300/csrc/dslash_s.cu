// Dispatch of the PrecS hopping kernels on isign.
#include "gbc_kernels.h"

namespace gbc {
int hop_launch_s0(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);
int hop_launch_s1(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s);
int hop_multi_launch_s0(int recon, int mode, int reduce, const HopArgs* args, const int2* work, int nwork,
                          cudaStream_t s);
int hop_multi_launch_s1(int recon, int mode, int reduce, const HopArgs* args, const int2* work, int nwork,
                          cudaStream_t s);
int hop_launch_s(int recon, int mode, bool dag, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  return dag ? hop_launch_s1(recon, mode, reduce, a, sh, s) : hop_launch_s0(recon, mode, reduce, a, sh, s);
}
int hop_multi_launch_s(int recon, int mode, bool dag, int reduce, const HopArgs* args, const int2* work, int nwork,
                         cudaStream_t s) {
  return dag ? hop_multi_launch_s1(recon, mode, reduce, args, work, nwork, s)
             : hop_multi_launch_s0(recon, mode, reduce, args, work, nwork, s);
}
}  // namespace gbc
