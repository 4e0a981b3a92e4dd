// Hopping kernels, storage precision PrecH, isign = PLUS.
#define GBC_RECON12 1
#include "dslash_inst.cuh"

namespace gbc {
int hop_launch_h0(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  return hop_recon<PrecH, false>(recon, mode, reduce, a, sh, s);
}
int hop_multi_launch_h0(int recon, int mode, int reduce, const HopArgs* args, const int2* work, int nwork,
                          cudaStream_t s) {
  return hop_multi_recon<PrecH, false>(recon, mode, reduce, args, work, nwork, s);
}
}  // namespace gbc
