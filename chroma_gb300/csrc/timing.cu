// gbc_time_operator: CUDA-event timing of the stencil kernels on device-resident fields.
#include "ctx.h"
#include "gbc_device.cuh"

namespace gbc {
namespace {

template <typename P>
__global__ void fill_kernel(Geom g, Spinor f, uint32_t seed) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (idx >= g.Vh) return;
  using T = typename P::real;
  cplx<T> v[12];
  uint32_t h = seed ^ (uint32_t)(idx * 2654435761u) ^ (uint32_t)(r * 40503u);
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    h = h * 1664525u + 1013904223u;
    T a = (T)((h >> 8) * (1.0 / 16777216.0) - 0.5);
    h = h * 1664525u + 1013904223u;
    T b = (T)((h >> 8) * (1.0 / 16777216.0) - 0.5);
    v[k] = {a, b};
  }
  store_spinor<P>((char*)f.v + (size_t)r * f.rhs_bytes, f.norm ? f.norm + (size_t)r * f.norm_rhs_stride : nullptr, idx,
                  g.stride, v);
}

__global__ void scribble(uint4* p, size_t n, uint32_t v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = make_uint4(v, v + 1, v + 2, v + 3);
}

void fill(gbc_ctx* c, const Spinor& f, uint32_t seed) {
  dim3 grid((c->g.Vh + 127) / 128, f.nrhs);
  if (f.prec == PREC_DOUBLE) fill_kernel<PrecD><<<grid, 128, 0, c->stream>>>(c->g, f, seed);
  else if (f.prec == PREC_SINGLE) fill_kernel<PrecS><<<grid, 128, 0, c->stream>>>(c->g, f, seed);
  else fill_kernel<PrecH><<<grid, 128, 0, c->stream>>>(c->g, f, seed);
}

}  // namespace

double link_bytes(int prec, int recon) { return (double)prec * (recon == 12 ? 12 : 18); }
double spinor_bytes(int prec) { return 24.0 * prec + (prec == PREC_HALF ? 4.0 : 0.0); }
double clover_site_bytes(int prec) { return 72.0 * prec; }

}  // namespace gbc

using namespace gbc;

extern "C" int gbc_time_operator(gbc_ctx* c, int op, int prec, int nrhs, int iters, int flush_l2, double* seconds,
                                 double* bytes) {
  if (!c || !seconds || iters < 1 || nrhs < 1 || nrhs > c->max_rhs) return GBC_ERR_ARGS;
  if (op != GBC_OP_DSLASH && op != GBC_OP_MEO && op != GBC_TIME_PRECOND) return GBC_ERR_ARGS;
  if (op == GBC_TIME_PRECOND && !c->precond) {
    c->err = "no learned preconditioner loaded";
    return GBC_ERR_PRECOND;
  }
  if (prec != GBC_PREC_DOUBLE && prec != GBC_PREC_SINGLE && prec != GBC_PREC_HALF && prec != GBC_PREC_DF64)
    return GBC_ERR_ARGS;
  if (prec == GBC_PREC_DF64 && op == GBC_TIME_PRECOND) return GBC_ERR_ARGS;
  const int sp = prec == GBC_PREC_DF64 ? GBC_PREC_DOUBLE : prec;  // storage of the fields
  if (!c->have_gauge) {
    c->err = "load the gauge field first";
    return GBC_ERR_STATE;
  }
  try {
    ensure_prec(c, prec);
    Spinor in = sub(workspace(c, 200, sp, nrhs), 0, nrhs);
    Spinor out = sub(workspace(c, 201, sp, nrhs), 0, nrhs);
    Spinor te = sub(workspace(c, 202, sp, nrhs), 0, nrhs);
    fill(c, in, 12345u);
    fill(c, out, 777u);
    uint4* junk = nullptr;
    const size_t junk_n = flush_l2 ? (256u << 20) / sizeof(uint4) : 0;
    if (flush_l2) GBC_CUDA(cudaMalloc(&junk, junk_n * sizeof(uint4)));
    cudaEvent_t e0, e1;
    GBC_CUDA(cudaEventCreate(&e0));
    GBC_CUDA(cudaEventCreate(&e1));
    double total = 0.0;
    auto launch = [&]() {
      if (op == GBC_OP_DSLASH) hop(c, prec, 1, HOP_PLAIN, false, 1.0, in, out, nullptr, nullptr, false);
      else if (op == GBC_OP_MEO) apply_meo(c, prec, false, in, out, te, false);
      else precond_apply(c, in, out);
    };
    launch();  // warm-up (module load, first-touch)
    for (int i = 0; i < iters; ++i) {
      if (flush_l2) scribble<<<152 * 4, 256, 0, c->stream>>>(junk, junk_n, (uint32_t)i);
      GBC_CUDA(cudaEventRecord(e0, c->stream));
      launch();
      GBC_CUDA(cudaEventRecord(e1, c->stream));
      GBC_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      GBC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      total += ms * 1e-3;
    }
    GBC_CUDA(cudaGetLastError());
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (junk) cudaFree(junk);
    *seconds = total / iters;
    if (bytes) {
      const PrecFields& f = c->pf[pidx(prec)];
      double L = link_bytes(sp, f.recon), S = spinor_bytes(sp), Cb = clover_site_bytes(sp);
      double Vh = c->g.Vh;
      if (op == GBC_TIME_PRECOND) {
        // per layer: the FP32 links of every site once, the FP32 activations in and out of every
        // right-hand side on both parities; plus the odd-site input and output spinors
        const double V = (double)c->V;
        double b = 2.0 * nrhs * Vh * S;
        for (int l = 0; l < precond_layers(c); ++l)
          b += V * 288.0 + nrhs * V * 24.0 * (precond_channels(c, l, false) + precond_channels(c, l, true));
        *bytes = b;
      } else {
        *bytes = op == GBC_OP_DSLASH ? Vh * (8 * L + 2.0 * nrhs * S) : Vh * (16 * L + 2 * Cb + 5.0 * nrhs * S);
      }
    }
    return GBC_OK;
  } catch (const CudaError& e) {
    c->err = std::string(e.where) + ": " + cudaGetErrorString(e.e);
    return GBC_ERR_CUDA;
  } catch (const std::string& s) {
    c->err = s;
    return GBC_ERR_STATE;
  }
}
