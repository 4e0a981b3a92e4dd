// Persistent batched CGNE with an FP32 stencil, both link reconstructions, and the dispatch over
// the precision pairs (FP64 sloppy batches have no persistent variant: per-launch path).
#define GBC_COHERENT_LOADS 1
#include "batch_persistent.cuh"
#include "ctx.h"

namespace gbc {

int batch_cg_persistent_h(int recon, const HopArgs* args, const LatCg* lat, const int2* work, int nwork, int n,
                          int kmax, double delta, PersistLat* pl, GridBar* bar, int* out, cudaStream_t s);

int batch_cg_persistent(int pa, int po, int recon, const HopArgs* args, const LatCg* lat, const int2* work,
                        int nwork, int n, int kmax, double delta, PersistLat* pl, GridBar* bar, int* out,
                        cudaStream_t s) {
  if (n < 1 || n > kPersistMaxLattices || pa != PREC_SINGLE || kmax < 1) return -1;
  int r = -1;
  if (po == PREC_HALF) r = batch_cg_persistent_h(recon, args, lat, work, nwork, n, kmax, delta, pl, bar, out, s);
  else if (po == PREC_SINGLE && recon == 12)
    r = persistent::launch<PrecS, PrecS, 12>(args, lat, work, nwork, n, kmax, delta, pl, bar, out, s);
  else if (po == PREC_SINGLE && recon == 18)
    r = persistent::launch<PrecS, PrecS, 18>(args, lat, work, nwork, n, kmax, delta, pl, bar, out, s);
  if (r == 0) count_launch();
  return r;
}

}  // namespace gbc
