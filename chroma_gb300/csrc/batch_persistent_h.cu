// Persistent batched CGNE with an fp16 stencil (FP32 accumulators), both link reconstructions.
#define GBC_COHERENT_LOADS 1
#include "batch_persistent.cuh"

namespace gbc {

int batch_cg_persistent_h(int recon, const HopArgs* args, const LatCg* lat, const int2* work, int nwork, int n,
                          int kmax, double delta, PersistLat* pl, GridBar* bar, int* out, cudaStream_t s) {
  if (recon == 12)
    return persistent::launch<PrecS, PrecH, 12>(args, lat, work, nwork, n, kmax, delta, pl, bar, out, s);
  if (recon == 18)
    return persistent::launch<PrecS, PrecH, 18>(args, lat, work, nwork, n, kmax, delta, pl, bar, out, s);
  return -1;
}

}  // namespace gbc
