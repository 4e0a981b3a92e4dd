// Synthetic gauge fields for benchmarks and tests (host, OpenMP): a seeded hot start
// U = reunit(exp(i eps H)) with H traceless Hermitian built from Gaussian entries, optional stout
// smearing (Chroma lib/util/gauge/stout_utils.cc:105-180, 936-966) and the time boundary sign
// (SimpleFermBC::modify, lib/actions/ferm/fermbcs/simple_fermbc.h:87-104).
//
// Random numbers are counter based, so the field does not depend on the thread count:
//   bits(seed, k)   = mix(mix(seed * 0x9E3779B97F4A7C15 + k)),  mix = the splitmix64 finaliser
//   uniform(seed,k) = ((bits >> 11) + 0.5) * 2^-53
//   normal(seed,k)  = sqrt(-2 ln uniform(seed, 2k)) cos(2 pi uniform(seed, 2k+1))
//   G[s][mu][row][col] = normal(base + 2e) + i normal(base + 2e + 1), base = (s*4+mu)*18, e = 3 row + col
//   H = (G + G^dag)/2 - tr/3
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/gbclover.h"

namespace {

using cd = std::complex<double>;

struct Mat {
  cd m[9];
};

Mat mul(const Mat& a, const Mat& b) {
  Mat r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
  return r;
}
Mat adj(const Mat& a) {
  Mat r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.m[3 * i + j] = std::conj(a.m[3 * j + i]);
  return r;
}
Mat eye() {
  Mat r;
  for (auto& x : r.m) x = 0.0;
  r.m[0] = r.m[4] = r.m[8] = 1.0;
  return r;
}

// exp(A) by scaling and squaring of a degree-18 Taylor polynomial
Mat expm(const Mat& a) {
  double nrm = 0;
  for (int i = 0; i < 3; ++i) {
    double s = std::abs(a.m[3 * i]) + std::abs(a.m[3 * i + 1]) + std::abs(a.m[3 * i + 2]);
    nrm = std::max(nrm, s);
  }
  int sq = 0;
  while (nrm > 0.25) {
    nrm *= 0.5;
    ++sq;
  }
  Mat as = a;
  double f = std::ldexp(1.0, -sq);
  for (auto& x : as.m) x *= f;
  Mat term = eye(), sum = eye();
  for (int k = 1; k <= 18; ++k) {
    term = mul(term, as);
    for (auto& x : term.m) x /= (double)k;
    for (int e = 0; e < 9; ++e) sum.m[e] += term.m[e];
  }
  for (int i = 0; i < sq; ++i) sum = mul(sum, sum);
  return sum;
}

// Gram-Schmidt on rows 0, 1; row 2 = conj(row0 x row1)  (lib/util/gauge/reunit.cc:205-262)
Mat reunit(Mat u) {
  double n0 = std::sqrt(std::norm(u.m[0]) + std::norm(u.m[1]) + std::norm(u.m[2]));
  for (int c = 0; c < 3; ++c) u.m[c] /= n0;
  cd ip = std::conj(u.m[0]) * u.m[3] + std::conj(u.m[1]) * u.m[4] + std::conj(u.m[2]) * u.m[5];
  for (int c = 0; c < 3; ++c) u.m[3 + c] -= ip * u.m[c];
  double n1 = std::sqrt(std::norm(u.m[3]) + std::norm(u.m[4]) + std::norm(u.m[5]));
  for (int c = 0; c < 3; ++c) u.m[3 + c] /= n1;
  u.m[6] = std::conj(u.m[1] * u.m[5] - u.m[2] * u.m[4]);
  u.m[7] = std::conj(u.m[2] * u.m[3] - u.m[0] * u.m[5]);
  u.m[8] = std::conj(u.m[0] * u.m[4] - u.m[1] * u.m[3]);
  return u;
}

inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
inline double uniform(uint64_t seed, uint64_t k) {
  return ((double)(mix64(mix64(seed * 0x9E3779B97F4A7C15ULL + k)) >> 11) + 0.5) * 0x1.0p-53;
}
inline double normal(uint64_t seed, uint64_t k) {
  return std::sqrt(-2.0 * std::log(uniform(seed, 2 * k))) * std::cos(6.283185307179586476925286766559 * uniform(seed, 2 * k + 1));
}

// exp(iQ) for traceless Hermitian Q: Cayley-Hamilton (Morningstar & Peardon, PRD 69 (2004) 054501)
Mat exp_iq(const Mat& Q) {
  Mat QQ = mul(Q, Q);
  double c0 = std::real(mul(QQ, Q).m[0] + mul(QQ, Q).m[4] + mul(QQ, Q).m[8]) / 3.0;
  double c1 = std::real(QQ.m[0] + QQ.m[4] + QQ.m[8]) / 2.0;
  if (c1 < 4e-3) {
    Mat iq = Q;
    for (auto& x : iq.m) x *= cd(0, 1);
    return expm(iq);
  }
  bool neg = c0 < 0;
  double c0max = 2.0 * std::pow(c1 / 3.0, 1.5);
  double theta = std::acos(std::min(1.0, std::fabs(c0) / c0max));
  double u = std::sqrt(c1 / 3.0) * std::cos(theta / 3.0), w = std::sqrt(c1) * std::sin(theta / 3.0);
  double u2 = u * u, w2 = w * w;
  double xi0 = std::fabs(w) < 0.05 ? 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0)) : std::sin(w) / w;
  double cw = std::cos(w);
  cd e2 = std::exp(cd(0, 2 * u)), em = std::exp(cd(0, -u));
  cd h0 = (u2 - w2) * e2 + em * (8.0 * u2 * cw + cd(0, 2.0 * u * (3.0 * u2 + w2)) * xi0);
  cd h1 = 2.0 * u * e2 - em * (2.0 * u * cw - cd(0, 3.0 * u2 - w2) * xi0);
  cd h2 = e2 - em * (cw + cd(0, 3.0 * u) * xi0);
  double den = 1.0 / (9.0 * u2 - w2);
  cd f0 = h0 * den, f1 = h1 * den, f2 = h2 * den;
  if (neg) {
    f0 = std::conj(f0);
    f1 = -std::conj(f1);
    f2 = std::conj(f2);
  }
  Mat r;
  for (int e = 0; e < 9; ++e) r.m[e] = f1 * Q.m[e] + f2 * QQ.m[e];
  r.m[0] += f0;
  r.m[4] += f0;
  r.m[8] += f0;
  return r;
}

struct Lat {
  int L[4];
  long V;
  long nb(long s, int mu, int d) const {
    int x[4];
    long r = s;
    for (int m = 0; m < 4; ++m) {
      x[m] = (int)(r % L[m]);
      r /= L[m];
    }
    x[mu] = (x[mu] + d + L[mu]) % L[mu];
    return x[0] + (long)L[0] * (x[1] + (long)L[1] * (x[2] + (long)L[2] * x[3]));
  }
};

Mat ld(const std::vector<Mat>& u, long s, int mu) { return u[s * 4 + mu]; }

void stout_step(const Lat& lat, const std::vector<Mat>& cur, std::vector<Mat>& nxt, double rho, const int* dirs) {
#pragma omp parallel for schedule(static)
  for (long s = 0; s < lat.V; ++s)
    for (int mu = 0; mu < 4; ++mu) {
      Mat U = ld(cur, s, mu);
      if (!dirs[mu]) {
        nxt[s * 4 + mu] = U;
        continue;
      }
      Mat C;
      for (auto& x : C.m) x = 0.0;
      for (int nu = 0; nu < 4; ++nu) {
        if (nu == mu || !dirs[nu]) continue;
        long xpm = lat.nb(s, mu, 1), xpn = lat.nb(s, nu, 1), xmn = lat.nb(s, nu, -1);
        long xmn_pm = lat.nb(xmn, mu, 1);
        Mat a = mul(mul(ld(cur, s, nu), ld(cur, xpn, mu)), adj(ld(cur, xpm, nu)));
        Mat b = mul(mul(adj(ld(cur, xmn, nu)), ld(cur, xmn, mu)), ld(cur, xmn_pm, nu));
        for (int e = 0; e < 9; ++e) C.m[e] += rho * (a.m[e] + b.m[e]);
      }
      Mat Om = mul(C, adj(U));
      Mat t = adj(Om);
      for (int e = 0; e < 9; ++e) t.m[e] -= Om.m[e];
      cd tr = (t.m[0] + t.m[4] + t.m[8]) / 3.0;
      t.m[0] -= tr;
      t.m[4] -= tr;
      t.m[8] -= tr;
      Mat Q;
      for (int e = 0; e < 9; ++e) Q.m[e] = cd(0, 0.5) * t.m[e];
      nxt[s * 4 + mu] = mul(exp_iq(Q), U);
    }
}

}  // namespace

extern "C" int gbc_gauge_synthetic(const int dims[4], double eps, unsigned long long seed, int n_stout, double rho,
                                   const int smear_dirs[4], int t_boundary, double* links) {
  if (!dims || !links) return GBC_ERR_ARGS;
  Lat lat;
  lat.V = 1;
  for (int m = 0; m < 4; ++m) {
    if (dims[m] < 1) return GBC_ERR_ARGS;
    lat.L[m] = dims[m];
    lat.V *= dims[m];
  }
  std::vector<Mat> u(lat.V * 4);
#pragma omp parallel for schedule(static)
  for (long s = 0; s < lat.V; ++s)
    for (int mu = 0; mu < 4; ++mu) {
      Mat G;
      uint64_t base = ((uint64_t)s * 4 + mu) * 18;
      for (int e = 0; e < 9; ++e) G.m[e] = cd(normal(seed, base + 2 * e), normal(seed, base + 2 * e + 1));
      Mat H;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H.m[3 * i + j] = 0.5 * (G.m[3 * i + j] + std::conj(G.m[3 * j + i]));
      cd tr = (H.m[0] + H.m[4] + H.m[8]) / 3.0;
      H.m[0] -= tr;
      H.m[4] -= tr;
      H.m[8] -= tr;
      for (auto& x : H.m) x *= cd(0, eps);
      u[s * 4 + mu] = reunit(expm(H));
    }
  const int all[4] = {1, 1, 1, 1};
  const int* dirs = smear_dirs ? smear_dirs : all;
  if (n_stout > 0) {
    std::vector<Mat> nxt(u.size());
    for (int i = 0; i < n_stout; ++i) {
      stout_step(lat, u, nxt, rho, dirs);
      u.swap(nxt);
    }
  }
  cd* out = reinterpret_cast<cd*>(links);
#pragma omp parallel for schedule(static)
  for (long s = 0; s < lat.V; ++s) {
    long t = s / ((long)lat.L[0] * lat.L[1] * lat.L[2]);
    for (int mu = 0; mu < 4; ++mu) {
      double f = (mu == 3 && t == lat.L[3] - 1 && t_boundary == -1) ? -1.0 : 1.0;
      for (int e = 0; e < 9; ++e) out[(s * 4 + mu) * 9 + e] = f * u[s * 4 + mu].m[e];
    }
  }
  return GBC_OK;
}
