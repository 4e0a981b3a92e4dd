// Clover term construction on the device, FP64, one thread per site:
//   F_{mu nu} = (1/8) (Q - Q^dag), Q = sum of the four plaquette leaves   (Chroma mesfield.cc:30-78)
//   A = diag_mass - sum_{mu<nu} c_{mu nu} gamma_mu gamma_nu F_{mu nu}, packed as Chroma's
//       PrimitiveClovTriang {diag[2][6], offd[2][15]}           (clover_term_qdp_w.h:244-294, 398-553)
//   A^-1 by LDL^dag factorisation of each 6x6 block + log|d_i| (clover_term_qdp_w.h:608-846)
#include "gbc_device.cuh"

namespace gbc {

namespace {

struct DM3 {
  cplx<double> a[9];
};

__device__ __forceinline__ DM3 dload(const double2* canon, long s, int mu) {
  DM3 m;
  const double2* p = canon + (s * 4 + mu) * 9;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    double2 v = p[k];
    m.a[k] = {v.x, v.y};
  }
  return m;
}
__device__ __forceinline__ DM3 dmul(const DM3& x, const DM3& y) {
  DM3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<double> v = x.a[3 * i] * y.a[j];
      cmac(v, x.a[3 * i + 1], y.a[3 + j]);
      cmac(v, x.a[3 * i + 2], y.a[6 + j]);
      r.a[3 * i + j] = v;
    }
  return r;
}
// x * y^dag
__device__ __forceinline__ DM3 dmul_nd(const DM3& x, const DM3& y) {
  DM3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<double> v = x.a[3 * i] * conj(y.a[3 * j]);
      cmac(v, x.a[3 * i + 1], conj(y.a[3 * j + 1]));
      cmac(v, x.a[3 * i + 2], conj(y.a[3 * j + 2]));
      r.a[3 * i + j] = v;
    }
  return r;
}
// x^dag * y
__device__ __forceinline__ DM3 dmul_dn(const DM3& x, const DM3& y) {
  DM3 r;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      cplx<double> v = conj(x.a[i]) * y.a[j];
      cmac(v, conj(x.a[3 + i]), y.a[3 + j]);
      cmac(v, conj(x.a[6 + i]), y.a[6 + j]);
      r.a[3 * i + j] = v;
    }
  return r;
}

__device__ __forceinline__ long shift_site(const int* L, const int* x, int mu, int d, int nu = -1, int e = 0) {
  int y[4] = {x[0], x[1], x[2], x[3]};
  y[mu] = (y[mu] + d + L[mu]) % L[mu];
  if (nu >= 0) y[nu] = (y[nu] + e + L[nu]) % L[nu];
  return y[0] + (long)L[0] * (y[1] + (long)L[1] * (y[2] + (long)L[2] * y[3]));
}

struct Dims {
  int L[4];
};

// LDL^dag factorisation and inverse of one packed 6x6 block in place (diag d[6], offd o[15]);
// accumulates log|d_i| and the count of negative d_i.
__device__ void ldl_invert_block(double* d, cplx<double>* o, double& logdet, int& nneg) {
  const int N = 6;
  cplx<double> v[6];
  for (int j = 0; j < N; ++j) {
    for (int i = 0; i < j; ++i) v[i] = d[i] * conj(o[j * (j - 1) / 2 + i]);
    v[j] = {d[j], 0.0};
    for (int k = 0; k < j; ++k) v[j] = v[j] - o[j * (j - 1) / 2 + k] * v[k];
    d[j] = v[j].re;
    const double inv = 1.0 / v[j].re;
    for (int k = j + 1; k < N; ++k) {
      const int ekj = k * (k - 1) / 2 + j;
      for (int l = 0; l < j; ++l) o[ekj] = o[ekj] - o[k * (k - 1) / 2 + l] * v[l];
      o[ekj] = inv * o[ekj];
    }
  }
  double dg[6];
  for (int i = 0; i < N; ++i) {
    dg[i] = 1.0 / d[i];
    logdet += log(fabs(d[i]));
    if (d[i] < 0) ++nneg;
  }
  double inv_d[6];
  cplx<double> inv_o[15];
  for (int k = 0; k < N; ++k) {
    for (int i = 0; i < k; ++i) v[i] = {0.0, 0.0};
    v[k] = {dg[k], 0.0};
    for (int i = k + 1; i < N; ++i) {
      cplx<double> acc = {0.0, 0.0};
      for (int j = k; j < i; ++j) acc = acc - d[j] * (o[i * (i - 1) / 2 + j] * v[j]);
      v[i] = dg[i] * acc;
    }
    for (int i = N - 2; i >= k; --i)
      for (int j = i + 1; j < N; ++j) v[i] = v[i] - conj(o[j * (j - 1) / 2 + i]) * v[j];
    inv_d[k] = v[k].re;
    for (int i = k + 1; i < N; ++i) inv_o[i * (i - 1) / 2 + k] = v[i];
  }
  for (int i = 0; i < N; ++i) d[i] = inv_d[i];
  for (int i = 0; i < 15; ++i) o[i] = inv_o[i];
}

__global__ void clover_build_kernel(Dims D, const double2* canon, CloverCoeffs cc, double* clov, double* inv,
                                    double* logdet, int* nneg, int inv_parity, long V) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= V) return;
  int x[4];
  {
    long r = s;
    x[0] = (int)(r % D.L[0]); r /= D.L[0];
    x[1] = (int)(r % D.L[1]); r /= D.L[1];
    x[2] = (int)(r % D.L[2]);
    x[3] = (int)(r / D.L[2]);
  }
  double diag[2][6];
  cplx<double> offd[2][15];
  for (int b = 0; b < 2; ++b)
    for (int i = 0; i < 6; ++i) diag[b][i] = cc.diag_mass;
  DM3 F[6];
  int k = 0;
  for (int mu = 0; mu < 3; ++mu)
    for (int nu = mu + 1; nu < 4; ++nu, ++k) {
      const long xpm = shift_site(D.L, x, mu, 1), xpn = shift_site(D.L, x, nu, 1);
      const long xmm = shift_site(D.L, x, mu, -1), xmn = shift_site(D.L, x, nu, -1);
      const long xmm_pn = shift_site(D.L, x, mu, -1, nu, 1), xmm_mn = shift_site(D.L, x, mu, -1, nu, -1);
      const long xmn_pm = shift_site(D.L, x, nu, -1, mu, 1);
      // U_1 = u(x,mu) u(x+mu,nu) u^dag(x+nu,mu) u^dag(x,nu)
      DM3 q = dmul_nd(dmul_nd(dmul(dload(canon, s, mu), dload(canon, xpm, nu)), dload(canon, xpn, mu)), dload(canon, s, nu));
      // U_2 = u(x,nu) u^dag(x-mu+nu,mu) u^dag(x-mu,nu) u(x-mu,mu)
      DM3 t = dmul(dmul_nd(dmul_nd(dload(canon, s, nu), dload(canon, xmm_pn, mu)), dload(canon, xmm, nu)), dload(canon, xmm, mu));
#pragma unroll
      for (int e = 0; e < 9; ++e) q.a[e] = q.a[e] + t.a[e];
      // U_3 = u^dag(x-mu,mu) u^dag(x-mu-nu,nu) u(x-mu-nu,mu) u(x-nu,nu)
      {
        // u^dag(x-mu,mu) u^dag(x-mu-nu,nu) = (u(x-mu-nu,nu) u(x-mu,mu))^dag
        DM3 w = dmul(dload(canon, xmm_mn, nu), dload(canon, xmm, mu));
        DM3 tail = dmul(dload(canon, xmm_mn, mu), dload(canon, xmn, nu));
        t = dmul_dn(w, tail);
      }
#pragma unroll
      for (int e = 0; e < 9; ++e) q.a[e] = q.a[e] + t.a[e];
      // U_4 = u^dag(x-nu,nu) u(x-nu,mu) u(x-nu+mu,nu) u^dag(x,mu)
      t = dmul_nd(dmul(dmul_dn(dload(canon, xmn, nu), dload(canon, xmn, mu)), dload(canon, xmn_pm, nu)), dload(canon, s, mu));
#pragma unroll
      for (int e = 0; e < 9; ++e) q.a[e] = q.a[e] + t.a[e];
      const double f = 0.125 * cc.coef[k];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F[k].a[3 * i + j] = f * (q.a[3 * i + j] - conj(q.a[3 * j + i]));
    }
  // makeClov (clover_term_qdp_w.h:398-553): F[0..5] = planes 01,02,03,12,13,23
  for (int i = 0; i < 3; ++i) {
    double r0 = (F[5].a[4 * i] - F[0].a[4 * i]).im;
    diag[0][i] += r0;
    diag[0][i + 3] -= r0;
    double r1 = (F[5].a[4 * i] + F[0].a[4 * i]).im;
    diag[1][i] -= r1;
    diag[1][i + 3] += r1;
  }
  for (int i = 1; i < 3; ++i)
    for (int j = 0; j < i; ++j) {
      int eij = i * (i - 1) / 2 + j;
      int etmp = (i + 3) * (i + 2) / 2 + j + 3;
      offd[0][eij] = timesI(F[0].a[3 * i + j] - F[5].a[3 * i + j]);
      offd[0][etmp] = -offd[0][eij];
      offd[1][eij] = timesI(F[5].a[3 * i + j] + F[0].a[3 * i + j]);
      offd[1][etmp] = -offd[1][eij];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      int eij = (i + 3) * (i + 2) / 2 + j;
      cplx<double> Em = timesI(F[2].a[3 * i + j]) + F[4].a[3 * i + j];
      cplx<double> Bm = timesI(F[3].a[3 * i + j]) - F[1].a[3 * i + j];
      offd[0][eij] = Bm - Em;
      offd[1][eij] = Em + Bm;
    }
  double* out = clov + s * 72;
  for (int b = 0; b < 2; ++b)
    for (int i = 0; i < 6; ++i) out[6 * b + i] = diag[b][i];
  for (int b = 0; b < 2; ++b)
    for (int i = 0; i < 15; ++i) {
      out[12 + 30 * b + 2 * i] = offd[b][i].re;
      out[12 + 30 * b + 2 * i + 1] = offd[b][i].im;
    }
  double* io = inv + s * 72;
  const int par = (x[0] + x[1] + x[2] + x[3]) & 1;
  if (inv_parity != 2 && par != inv_parity) {
    for (int i = 0; i < 72; ++i) io[i] = 0.0;
    logdet[s] = 0.0;
    nneg[s] = 0;
    return;
  }
  double ld = 0.0;
  int nn = 0;
  for (int b = 0; b < 2; ++b) ldl_invert_block(diag[b], offd[b], ld, nn);
  for (int b = 0; b < 2; ++b)
    for (int i = 0; i < 6; ++i) io[6 * b + i] = diag[b][i];
  for (int b = 0; b < 2; ++b)
    for (int i = 0; i < 15; ++i) {
      io[12 + 30 * b + 2 * i] = offd[b][i].re;
      io[12 + 30 * b + 2 * i + 1] = offd[b][i].im;
    }
  logdet[s] = ld;
  nneg[s] = nn;
}

__global__ void clover_invert_kernel(long n, double* packed, double* logdet, int* nneg) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  double* p = packed + s * 72;
  double d[2][6];
  cplx<double> o[2][15];
  for (int b = 0; b < 2; ++b) {
    for (int i = 0; i < 6; ++i) d[b][i] = p[6 * b + i];
    for (int i = 0; i < 15; ++i) o[b][i] = {p[12 + 30 * b + 2 * i], p[13 + 30 * b + 2 * i]};
  }
  double ld = 0.0;
  int nn = 0;
  for (int b = 0; b < 2; ++b) ldl_invert_block(d[b], o[b], ld, nn);
  for (int b = 0; b < 2; ++b) {
    for (int i = 0; i < 6; ++i) p[6 * b + i] = d[b][i];
    for (int i = 0; i < 15; ++i) {
      p[12 + 30 * b + 2 * i] = o[b][i].re;
      p[13 + 30 * b + 2 * i] = o[b][i].im;
    }
  }
  logdet[s] = ld;
  nneg[s] = nn;
}

}  // namespace

void clover_build(const int dims[4], const double* canon_links, const CloverCoeffs& cc, double* clov, double* inv,
                  double* logdet, int* nneg, int inv_parity, cudaStream_t s) {
  Dims D{{dims[0], dims[1], dims[2], dims[3]}};
  long V = (long)dims[0] * dims[1] * dims[2] * dims[3];
  clover_build_kernel<<<(unsigned)((V + 63) / 64), 64, 0, s>>>(D, reinterpret_cast<const double2*>(canon_links), cc,
                                                               clov, inv, logdet, nneg, inv_parity, V);
}

// inv = A^-1 on the sites of parity `parity` (clov on all sites, canonical site order)
__global__ void clover_invert_parity_kernel(Dims D, const double* clov, double* inv, int parity, long V) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= V) return;
  long r = s;
  int sum = 0;
  for (int k = 0; k < 4; ++k) {
    sum += (int)(r % D.L[k]);
    r /= D.L[k];
  }
  if ((sum & 1) != parity) return;
  const double* p = clov + s * 72;
  double* q = inv + s * 72;
  double d[2][6];
  cplx<double> o[2][15];
  for (int b = 0; b < 2; ++b) {
    for (int i = 0; i < 6; ++i) d[b][i] = p[6 * b + i];
    for (int i = 0; i < 15; ++i) o[b][i] = {p[12 + 30 * b + 2 * i], p[13 + 30 * b + 2 * i]};
  }
  double ld = 0.0;
  int nn = 0;
  for (int b = 0; b < 2; ++b) ldl_invert_block(d[b], o[b], ld, nn);
  for (int b = 0; b < 2; ++b) {
    for (int i = 0; i < 6; ++i) q[6 * b + i] = d[b][i];
    for (int i = 0; i < 15; ++i) {
      q[12 + 30 * b + 2 * i] = o[b][i].re;
      q[13 + 30 * b + 2 * i] = o[b][i].im;
    }
  }
}

void clover_invert(long nsites, double* packed, double* logdet, int* nneg, cudaStream_t s) {
  clover_invert_kernel<<<(unsigned)((nsites + 63) / 64), 64, 0, s>>>(nsites, packed, logdet, nneg);
}

void clover_invert_parity(const int dims[4], const double* clov, double* inv, int parity, cudaStream_t s) {
  Dims D{{dims[0], dims[1], dims[2], dims[3]}};
  long V = (long)dims[0] * dims[1] * dims[2] * dims[3];
  clover_invert_parity_kernel<<<(unsigned)((V + 63) / 64), 64, 0, s>>>(D, clov, inv, parity, V);
}

}  // namespace gbc
