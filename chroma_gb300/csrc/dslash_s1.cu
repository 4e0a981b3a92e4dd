// Hopping kernels, storage precision PrecS, isign = MINUS (dagger).
#define GBC_RECON12 1
#include "dslash_inst.cuh"

namespace gbc {
int hop_launch_s1(int recon, int mode, int reduce, const HopArgs& a, HopShape sh, cudaStream_t s) {
  return hop_recon<PrecS, true>(recon, mode, reduce, a, sh, s);
}
int hop_multi_launch_s1(int recon, int mode, int reduce, const HopArgs* args, const int2* work, int nwork,
                          cudaStream_t s) {
  return hop_multi_recon<PrecS, true>(recon, mode, reduce, args, work, nwork, s);
}
}  // namespace gbc
