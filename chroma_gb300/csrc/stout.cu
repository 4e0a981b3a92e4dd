// Stout smearing of the gauge field on the device, FP64 (setup of smeared-link actions).
//
//   C_mu(x) = rho sum_{nu != mu, smeared} [ U_nu(x) U_mu(x+nu) U_nu^dag(x+mu)
//                                          + U_nu^dag(x-nu) U_mu(x-nu) U_nu(x-nu+mu) ]
//   Omega = C U^dag,  Q = (i/2) (Omega^dag - Omega) - (i/6) tr(Omega^dag - Omega),
//   U'_mu(x) = exp(i Q) U_mu(x)
// (Chroma lib/util/gauge/stout_utils.cc:105-180 getQsandCs, :936-966 smear_links), with exp(iQ)
// by the Cayley-Hamilton form of Morningstar & Peardon, PRD 69 (2004) 054501 (stout_utils.cc:
// 415-700), and for tr(Q^2)/2 < 4e-3 a scaled-and-squared Taylor series of exp(iQ).
//
// One thread per link (site, mu) of the canonical layout [V][4][3][3] complex; the staples read
// their links through L1/L2 (each link is read by up to 18 staples).  Links of directions that are
// not smeared are copied.
#include <cuda_runtime.h>

#include <string>

#include "ctx.h"

namespace gbc {
namespace {

struct M {
  double2 a[9];
};

__device__ __forceinline__ double2 cm(double2 x, double2 y) { return make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x); }
__device__ __forceinline__ double2 cadd(double2 x, double2 y) { return make_double2(x.x + y.x, x.y + y.y); }
__device__ __forceinline__ double2 cs(double2 x, double2 f) { return cm(x, f); }

__device__ __forceinline__ M mmul(const M& x, const M& y) {
  M r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      r.a[3 * i + j] = cadd(cadd(cm(x.a[3 * i], y.a[j]), cm(x.a[3 * i + 1], y.a[3 + j])), cm(x.a[3 * i + 2], y.a[6 + j]));
  return r;
}
__device__ __forceinline__ M madj(const M& x) {
  M r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) r.a[3 * i + j] = make_double2(x.a[3 * j + i].x, -x.a[3 * j + i].y);
  return r;
}
__device__ __forceinline__ M mone() {
  M r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.a[k] = make_double2(k % 4 == 0 ? 1.0 : 0.0, 0.0);
  return r;
}
__device__ __forceinline__ M madd(const M& x, const M& y) {
  M r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.a[k] = cadd(x.a[k], y.a[k]);
  return r;
}
__device__ __forceinline__ M mscale(const M& x, double2 f) {
  M r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.a[k] = cs(x.a[k], f);
  return r;
}
__device__ __forceinline__ double2 mtrace(const M& x) { return cadd(cadd(x.a[0], x.a[4]), x.a[8]); }
__device__ __forceinline__ M ld(const double2* u, long site, int mu) {
  M r;
  const double2* p = u + (site * 4 + mu) * 9;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.a[k] = p[k];
  return r;
}

// exp(A), general 3x3: scaling by 2^-s until the max row sum is <= 1/4, 18 Taylor terms, s squarings
__device__ M mexp_taylor(const M& A) {
  double nrm = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double r = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) r += hypot(A.a[3 * i + j].x, A.a[3 * i + j].y);
    nrm = fmax(nrm, r);
  }
  int sq = 0;
  while (nrm > 0.25 && sq < 60) {
    nrm *= 0.5;
    ++sq;
  }
  const M As = mscale(A, make_double2(ldexp(1.0, -sq), 0.0));
  M term = mone(), sum = mone();
  for (int k = 1; k <= 18; ++k) {
    term = mscale(mmul(term, As), make_double2(1.0 / k, 0.0));
    sum = madd(sum, term);
  }
  for (int i = 0; i < sq; ++i) sum = mmul(sum, sum);
  return sum;
}

// exp(iQ) for traceless Hermitian Q: f0 + f1 Q + f2 Q^2 (Morningstar-Peardon)
__device__ M exp_iQ(const M& Q) {
  const M QQ = mmul(Q, Q);
  const double c0 = mtrace(mmul(QQ, Q)).x / 3.0;
  const double c1 = mtrace(QQ).x / 2.0;
  if (c1 < 4.0e-3) return mexp_taylor(mscale(Q, make_double2(0.0, 1.0)));
  const bool neg = c0 < 0;
  const double c0a = fabs(c0);
  const double c0max = 2.0 * pow(c1 / 3.0, 1.5);
  const double theta = acos(fmin(1.0, c0a / c0max));
  const double u = sqrt(c1 / 3.0) * cos(theta / 3.0);
  const double w = sqrt(c1) * sin(theta / 3.0);
  const double u2 = u * u, w2 = w * w;
  const double xi0 = fabs(w) < 0.05 ? 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0)) : sin(w) / w;
  const double cw = cos(w);
  double s2u, c2u, su, cu;
  sincos(2.0 * u, &s2u, &c2u);
  sincos(u, &su, &cu);
  const double2 e2iu = make_double2(c2u, s2u), emiu = make_double2(cu, -su);
  // h0 = (u2 - w2) e2iu + emiu (8 u2 cw + 2i u (3u2 + w2) xi0)
  double2 h0 = cadd(make_double2((u2 - w2) * e2iu.x, (u2 - w2) * e2iu.y),
                    cm(emiu, make_double2(8.0 * u2 * cw, 2.0 * u * (3.0 * u2 + w2) * xi0)));
  // h1 = 2u e2iu - emiu (2u cw - i (3u2 - w2) xi0)
  double2 t1 = cm(emiu, make_double2(2.0 * u * cw, -(3.0 * u2 - w2) * xi0));
  double2 h1 = make_double2(2.0 * u * e2iu.x - t1.x, 2.0 * u * e2iu.y - t1.y);
  // h2 = e2iu - emiu (cw + 3i u xi0)
  double2 t2 = cm(emiu, make_double2(cw, 3.0 * u * xi0));
  double2 h2 = make_double2(e2iu.x - t2.x, e2iu.y - t2.y);
  const double den = 1.0 / (9.0 * u2 - w2);
  double2 f0 = make_double2(h0.x * den, h0.y * den), f1 = make_double2(h1.x * den, h1.y * den),
          f2 = make_double2(h2.x * den, h2.y * den);
  if (neg) {
    f0.y = -f0.y;
    f1.x = -f1.x;
    f2.y = -f2.y;
  }
  M r = mscale(mone(), f0);
  r = madd(r, mscale(Q, f1));
  r = madd(r, mscale(QQ, f2));
  return r;
}

struct Lat {
  int L[4];
  long V;
};

__device__ __forceinline__ long shift(const Lat& g, long s, int mu, int d) {
  int x[4];
  long r = s;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    x[k] = (int)(r % g.L[k]);
    r /= g.L[k];
  }
  x[mu] = (x[mu] + d + g.L[mu]) % g.L[mu];
  return x[0] + (long)g.L[0] * (x[1] + (long)g.L[1] * (x[2] + (long)g.L[2] * x[3]));
}

__global__ void __launch_bounds__(128) stout_kernel(Lat g, const double2* __restrict__ cur, double2* __restrict__ nxt,
                                                    double rho, int4 dirs) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.V * 4) return;
  const long s = t >> 2;
  const int mu = (int)(t & 3);
  const int on[4] = {dirs.x, dirs.y, dirs.z, dirs.w};
  const M U = ld(cur, s, mu);
  M out = U;
  if (on[mu]) {
    M C;
#pragma unroll
    for (int k = 0; k < 9; ++k) C.a[k] = make_double2(0.0, 0.0);
    const long sp_mu = shift(g, s, mu, +1);
    for (int nu = 0; nu < 4; ++nu) {
      if (nu == mu || !on[nu]) continue;
      const long sp_nu = shift(g, s, nu, +1), sm_nu = shift(g, s, nu, -1);
      const long sm_nu_p_mu = shift(g, sm_nu, mu, +1);
      M st = mmul(mmul(ld(cur, s, nu), ld(cur, sp_nu, mu)), madj(ld(cur, sp_mu, nu)));
      st = madd(st, mmul(mmul(madj(ld(cur, sm_nu, nu)), ld(cur, sm_nu, mu)), ld(cur, sm_nu_p_mu, nu)));
      C = madd(C, mscale(st, make_double2(rho, 0.0)));
    }
    const M Om = mmul(C, madj(U));
    const M Oa = madj(Om);
    M t2;
#pragma unroll
    for (int k = 0; k < 9; ++k) t2.a[k] = make_double2(Oa.a[k].x - Om.a[k].x, Oa.a[k].y - Om.a[k].y);
    const double2 tr = mtrace(t2);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      t2.a[4 * i].x -= tr.x / 3.0;
      t2.a[4 * i].y -= tr.y / 3.0;
    }
    const M Q = mscale(t2, make_double2(0.0, 0.5));
    out = mmul(exp_iQ(Q), U);
  }
  double2* p = nxt + (s * 4 + mu) * 9;
#pragma unroll
  for (int k = 0; k < 9; ++k) p[k] = out.a[k];
}

}  // namespace
}  // namespace gbc

using namespace gbc;

extern "C" int gbc_stout_smear(const gbc_geom* geom, int n_steps, double rho, const int smear_dirs[4],
                               const double* links_in, double* links_out) {
  if (!geom || !links_in || !links_out || n_steps < 0) return GBC_ERR_ARGS;
  Lat g;
  g.V = 1;
  for (int k = 0; k < 4; ++k) {
    if (geom->dims[k] < 2) return GBC_ERR_ARGS;
    g.L[k] = geom->dims[k];
    g.V *= geom->dims[k];
  }
  const int all[4] = {1, 1, 1, 1};
  const int* d = smear_dirs ? smear_dirs : all;
  const int4 dirs = make_int4(d[0] != 0, d[1] != 0, d[2] != 0, d[3] != 0);
  const size_t bytes = sizeof(double) * 72 * (size_t)g.V;
  double2* buf[2] = {nullptr, nullptr};
  cudaStream_t s = nullptr;
  int rc = GBC_OK;
  if (cudaMalloc(&buf[0], bytes) != cudaSuccess || cudaMalloc(&buf[1], bytes) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    rc = GBC_ERR_CUDA;
  } else {
    cudaMemcpyAsync(buf[0], links_in, bytes, cudaMemcpyHostToDevice, s);
    const long threads = g.V * 4;
    for (int i = 0; i < n_steps; ++i) {
      stout_kernel<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(g, buf[i & 1], buf[(i + 1) & 1], rho, dirs);
      count_launch();
    }
    cudaMemcpyAsync(links_out, buf[n_steps & 1], bytes, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = GBC_ERR_CUDA;
  }
  if (buf[0]) cudaFree(buf[0]);
  if (buf[1]) cudaFree(buf[1]);
  if (s) cudaStreamDestroy(s);
  return rc;
}
