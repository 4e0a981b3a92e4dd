// gbc_apply_meo_noalloc: the even-odd clover operator M~ in FP64 with no device allocation.
//
// Some callers cannot allocate device memory while they run.  Chroma built on QDP-JIT is the
// main one here: QDP-JIT's pool allocator reserves most of the GPU's memory when it starts, so a
// cudaMalloc issued later from a library may fail, and a cudaMalloc/cudaFree pair can also
// synchronise the device in the middle of a caller's pipelined stream work.  The ordinary entry
// points allocate their workspaces inside a gbc_ctx.  This one takes every input and output as a
// caller-owned device pointer in the canonical layouts of gbclover.h, and the only temporary it
// needs -- the even-parity intermediate A_ee^-1 D_eo psi_o -- lives in a file-scope static
// __device__ array of fixed size, which every GPU that loads the library holds until exit.
//
// The two kernels follow the same algebra as apply_meo (Chroma eoprec_clover_linop_w.cc:142-187)
// but read the canonical array-of-structures layout directly.
#include <cstdio>
#include <mutex>

#include "../../include/gbclover.h"
#include "dslash.cuh"

namespace gbc {
namespace {

// Even-parity intermediate, GBC_NOALLOC_MAX_VH sites x 12 complex doubles (12 MiB).
static __device__ __align__(256) double2 noalloc_scratch[(size_t)GBC_NOALLOC_MAX_VH * 12];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double2* g_scratch_ptr[kMaxDevices] = {nullptr};

struct CanonGeom {
  int L[4];
  int Lxh;
  int Vh;
};

__device__ __forceinline__ Coord cg_coords(const CanonGeom& g, int i, int parity) {
  Coord c;
  int xh = i % g.Lxh;
  int r = i / g.Lxh;
  c.x[1] = r % g.L[1];
  r /= g.L[1];
  c.x[2] = r % g.L[2];
  c.x[3] = r / g.L[2];
  c.x[0] = 2 * xh + ((parity + c.x[1] + c.x[2] + c.x[3]) & 1);
  return c;
}
__device__ __forceinline__ long cg_full(const CanonGeom& g, const Coord& c) {
  return c.x[0] + (long)g.L[0] * (c.x[1] + (long)g.L[1] * (c.x[2] + (long)g.L[2] * c.x[3]));
}
__device__ __forceinline__ int cg_half(const CanonGeom& g, const Coord& c) {
  return (c.x[0] >> 1) + g.Lxh * (c.x[1] + g.L[1] * (c.x[2] + g.L[2] * c.x[3]));
}

__device__ __forceinline__ void ld_site(cplx<double> (&v)[12], const double2* p) {
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    double2 w = p[k];
    v[k] = {w.x, w.y};
  }
}
__device__ __forceinline__ void ld_link(cplx<double> (&u)[9], const double2* p) {
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    double2 w = p[k];
    u[k] = {w.x, w.y};
  }
}
// y = T x for the two chiral blocks of one canonical packed site {diag[2][6], offd[2][15]}
__device__ __forceinline__ void clover_site(cplx<double> (&y)[12], const double* t, const cplx<double> (&x)[12]) {
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    double d[6];
    cplx<double> o[15], xb[6], yb[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) d[k] = t[6 * b + k];
#pragma unroll
    for (int k = 0; k < 15; ++k) o[k] = {t[12 + 30 * b + 2 * k], t[13 + 30 * b + 2 * k]};
#pragma unroll
    for (int k = 0; k < 6; ++k) xb[k] = x[6 * b + k];
    clover_block_mul(yb, d, o, xb);
#pragma unroll
    for (int k = 0; k < 6; ++k) y[6 * b + k] = yb[k];
  }
}

// D' psi at site c (parity of c), reading psi from the canonical array (other parity) or, for
// the second half, from the even scratch indexed by checkerboard index.
template <bool DAG, bool FROM_SCRATCH>
__device__ void hop_canon(cplx<double> (&acc)[12], const CanonGeom& g, const Coord& c, const double2* links,
                          const double2* psi, const double2* scratch) {
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[k] = {0.0, 0.0};
  cplx<double> s[12], h[2][3], uh[2][3], u[9];
  const long self = cg_full(g, c);
#pragma unroll
  for (int mu = 0; mu < 4; ++mu) {
    Coord n = c;
    n.x[mu] = c.x[mu] + 1 == g.L[mu] ? 0 : c.x[mu] + 1;
    if (FROM_SCRATCH) ld_site(s, scratch + (size_t)cg_half(g, n) * 12);
    else ld_site(s, psi + cg_full(g, n) * 12);
    ld_link(u, links + (self * 4 + mu) * 9);
    // forward: U(x) (1 - isign gamma) psi(x+mu)
    switch (mu) {
      case 0: project<0, DAG ? 1 : -1>(h, s); break;
      case 1: project<1, DAG ? 1 : -1>(h, s); break;
      case 2: project<2, DAG ? 1 : -1>(h, s); break;
      default: project<3, DAG ? 1 : -1>(h, s); break;
    }
    mat_vec2(uh, u, h);
    switch (mu) {
      case 0: reconstruct<0, DAG ? 1 : -1>(acc, uh); break;
      case 1: reconstruct<1, DAG ? 1 : -1>(acc, uh); break;
      case 2: reconstruct<2, DAG ? 1 : -1>(acc, uh); break;
      default: reconstruct<3, DAG ? 1 : -1>(acc, uh); break;
    }
    n.x[mu] = c.x[mu] == 0 ? g.L[mu] - 1 : c.x[mu] - 1;
    const long nb = cg_full(g, n);
    if (FROM_SCRATCH) ld_site(s, scratch + (size_t)cg_half(g, n) * 12);
    else ld_site(s, psi + nb * 12);
    ld_link(u, links + (nb * 4 + mu) * 9);
    // backward: U^dag(x-mu) (1 + isign gamma) psi(x-mu)
    switch (mu) {
      case 0: project<0, DAG ? -1 : 1>(h, s); break;
      case 1: project<1, DAG ? -1 : 1>(h, s); break;
      case 2: project<2, DAG ? -1 : 1>(h, s); break;
      default: project<3, DAG ? -1 : 1>(h, s); break;
    }
    adj_mat_vec2(uh, u, h);
    switch (mu) {
      case 0: reconstruct<0, DAG ? -1 : 1>(acc, uh); break;
      case 1: reconstruct<1, DAG ? -1 : 1>(acc, uh); break;
      case 2: reconstruct<2, DAG ? -1 : 1>(acc, uh); break;
      default: reconstruct<3, DAG ? -1 : 1>(acc, uh); break;
    }
  }
}

// even sites: scratch[cb] = A_ee^-1 D'_eo psi_o
template <bool DAG>
__global__ void noalloc_even(CanonGeom g, const double2* links, const double* invclov, const double2* psi,
                             double2* scratch) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.Vh) return;
  const Coord c = cg_coords(g, i, 0);
  cplx<double> acc[12], y[12];
  hop_canon<DAG, false>(acc, g, c, links, psi, nullptr);
  clover_site(y, invclov + cg_full(g, c) * 72, acc);
#pragma unroll
  for (int k = 0; k < 12; ++k) scratch[(size_t)i * 12 + k] = make_double2(y[k].re, y[k].im);
}

// odd sites: out = A_oo psi_o - 1/4 D'_oe scratch  (+ isign i mu gamma_5 psi_o)
template <bool DAG>
__global__ void noalloc_odd(CanonGeom g, const double2* links, const double* clov, const double2* psi,
                            const double2* scratch, double twist, double2* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.Vh) return;
  const Coord c = cg_coords(g, i, 1);
  const long s = cg_full(g, c);
  cplx<double> acc[12], x[12], y[12];
  hop_canon<DAG, true>(acc, g, c, links, nullptr, scratch);
  ld_site(x, psi + s * 12);
  clover_site(y, clov + s * 72, x);
  const double tw = DAG ? -twist : twist;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    cplx<double> v = y[k];
    v.re = fmadd(-0.25, acc[k].re, v.re);
    v.im = fmadd(-0.25, acc[k].im, v.im);
    if (twist != 0.0) v = v + (k < 6 ? tw : -tw) * timesI(x[k]);
    out[s * 12 + k] = make_double2(v.re, v.im);
  }
}

}  // namespace

// Device address of the scratch array on the current device; looked up once per device.  The
// lookup is also what makes the array exist there: under CUDA's default lazy module loading
// (CUDA_MODULE_LOADING=LAZY) this file's module, with its static array, is loaded on the first
// use of one of its symbols, not when the library is loaded.
int noalloc_scratch_for_current_device(double2** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GBC_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, noalloc_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "gbc_apply_meo_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
              cudaGetErrorString(e));
      return GBC_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<double2*>(p);
  }
  *out = g_scratch_ptr[dev];
  return GBC_OK;
}

int noalloc_reserve() {
  double2* p = nullptr;
  return noalloc_scratch_for_current_device(&p);
}

}  // namespace gbc

extern "C" int gbc_apply_meo_noalloc(const gbc_geom* geom, const gbc_action* act, const double* links_dev,
                                     const double* clov_dev, const double* invclov_dev, int isign, double* out_dev,
                                     const double* in_dev, void* stream) {
  using namespace gbc;
  if (!geom || !act || !links_dev || !clov_dev || !invclov_dev || !out_dev || !in_dev) return GBC_ERR_ARGS;
  if (isign != 1 && isign != -1) return GBC_ERR_ARGS;
  // every extent even: with an odd extent the wrap-around neighbour has the site's own parity
  for (int m = 0; m < 4; ++m)
    if (geom->dims[m] < 2 || geom->dims[m] % 2) return GBC_ERR_ARGS;
  const long V = (long)geom->dims[0] * geom->dims[1] * geom->dims[2] * geom->dims[3];
  if (V / 2 > GBC_NOALLOC_MAX_VH) {
    fprintf(stderr,
            "gbc_apply_meo_noalloc: %ld sites per checkerboard exceed the static scratch of %d; "
            "use gbc_apply for this lattice\n",
            V / 2, GBC_NOALLOC_MAX_VH);
    return GBC_ERR_ARGS;
  }
  double2* scratch = nullptr;
  int rc = noalloc_scratch_for_current_device(&scratch);
  if (rc != GBC_OK) return rc;
  CanonGeom g;
  for (int m = 0; m < 4; ++m) g.L[m] = geom->dims[m];
  g.Lxh = g.L[0] / 2;
  g.Vh = (int)(V / 2);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double2* links = reinterpret_cast<const double2*>(links_dev);
  const double2* in = reinterpret_cast<const double2*>(in_dev);
  double2* out = reinterpret_cast<double2*>(out_dev);
  const double twist = act->twisted ? act->twisted_m : 0.0;
  const int threads = 128;
  const unsigned blocks = (unsigned)((g.Vh + threads - 1) / threads);
  // the scratch is fully overwritten by the first kernel on every call: nothing to clear
  if (isign > 0) {
    noalloc_even<false><<<blocks, threads, 0, s>>>(g, links, invclov_dev, in, scratch);
    noalloc_odd<false><<<blocks, threads, 0, s>>>(g, links, clov_dev, in, scratch, twist, out);
  } else {
    noalloc_even<true><<<blocks, threads, 0, s>>>(g, links, invclov_dev, in, scratch);
    noalloc_odd<true><<<blocks, threads, 0, s>>>(g, links, clov_dev, in, scratch, twist, out);
  }
  return cudaGetLastError() == cudaSuccess ? GBC_OK : GBC_ERR_CUDA;
}
