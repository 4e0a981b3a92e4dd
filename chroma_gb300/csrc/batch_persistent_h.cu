// Persistent batched CGNE with an fp16 stencil (FP32 accumulators), both link reconstructions.
#define GBC_COHERENT_LOADS 1
#include "batch_persistent.cuh"

namespace gbc {

int batch_cg_persistent_h(int recon, const HopArgs* args, const LatCg* lat, const int2* work, int nwork, int n,
                          int kmax, double delta, PersistLat* pl, GridBar* bar, int* out, cudaStream_t s) {
  if (recon == 12) {
    // 3 resident blocks per SM (158 registers): measured 1.4 % faster than 4 (127) and 10 % faster
    // than 2 on the 20^3 x 40 ... 8^3 x 16 batch, no difference on small batches
    return persistent::launch<PrecS, PrecH, 12, 3>(args, lat, work, nwork, n, kmax, delta, pl, bar, out, s);
  }
  if (recon == 18)
    return persistent::launch<PrecS, PrecH, 18>(args, lat, work, nwork, n, kmax, delta, pl, bar, out, s);
  return -1;
}

}  // namespace gbc
