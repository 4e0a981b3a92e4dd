// CPU check of the small dense complex algebra of the FGMRES-DR restart (chroma_gb300/csrc/dense.cc):
// Schur form and reordering, LU solves, thin QR, and the harmonic-Ritz property the deflated
// restart relies on.  Exits non-zero on the first failed bound; prints one line per check.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>

#include "../../chroma_gb300/csrc/dense.h"

using namespace gbc::dense;

static int fails = 0;
static void check(bool ok, const char* what, int n, double v) {
  std::printf("%-34s n=%2d %.3e %s\n", what, n, v, ok ? "ok" : "FAIL");
  if (!ok) ++fails;
}

int main() {
  std::mt19937 rng(3);
  std::normal_distribution<double> nd;
  for (int n : {1, 2, 5, 17, 33}) {
    std::vector<cd> A((size_t)n * n), T, Q;
    for (auto& x : A) x = cd(nd(rng), nd(rng));
    T = A;
    const bool conv = schur(n, T, Q);
    check(conv, "schur converged", n, 0.0);
    const int k = std::min(n, 6);
    sort_smallest(n, T, Q, k);
    double err = 0, low = 0, un = 0, scale = 0;
    for (auto& x : A) scale = std::max(scale, std::abs(x));
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        cd s = 0;
        for (int p = 0; p < n; ++p)
          for (int q = 0; q < n; ++q) s += Q[(size_t)p * n + i] * T[(size_t)q * n + p] * std::conj(Q[(size_t)q * n + j]);
        err = std::max(err, std::abs(s - A[(size_t)j * n + i]));
        if (i > j) low = std::max(low, std::abs(T[(size_t)j * n + i]));
        cd u = 0;
        for (int p = 0; p < n; ++p) u += std::conj(Q[(size_t)i * n + p]) * Q[(size_t)j * n + p];
        un = std::max(un, std::abs(u - (i == j ? 1.0 : 0.0)));
      }
    check(err < 1e-12 * n * scale, "A = Q T Q^H", n, err);
    check(low == 0.0, "T upper triangular", n, low);
    check(un < 1e-13 * n, "Q unitary", n, un);
    std::vector<double> mods(n);
    for (int i = 0; i < n; ++i) mods[i] = std::abs(T[(size_t)i * n + i]);
    std::vector<double> srt = mods;
    std::sort(srt.begin(), srt.end());
    double dsort = 0;
    for (int i = 0; i < k; ++i) dsort = std::max(dsort, std::abs(mods[i] - srt[i]));
    check(dsort < 1e-10 * scale, "k smallest |eigenvalues| lead", n, dsort);
    std::vector<cd> b(n), x;
    for (auto& v : b) v = cd(nd(rng), nd(rng));
    for (int adj = 0; adj < 2; ++adj) {
      x = b;
      const bool ok = lu_solve(n, A, x, adj != 0);
      double r = 0;
      for (int i = 0; i < n; ++i) {
        cd s = 0;
        for (int j = 0; j < n; ++j) s += (adj ? std::conj(A[(size_t)i * n + j]) : A[(size_t)j * n + i]) * x[j];
        r = std::max(r, std::abs(s - b[i]));
      }
      check(ok && r < 1e-10, adj ? "LU solve A^H x = b" : "LU solve A x = b", n, r);
    }
  }
  // thin QR of a (d+1) x (k+1) matrix
  {
    const int m = 9, k = 4;
    std::vector<cd> G((size_t)m * k), R, G0;
    for (auto& x : G) x = cd(nd(rng), nd(rng));
    G0 = G;
    qr_thin(m, k, G, R);
    double e = 0, un = 0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < k; ++j) {
        cd s = 0;
        for (int q = 0; q < k; ++q) s += G[(size_t)q * m + i] * R[(size_t)j * k + q];
        e = std::max(e, std::abs(s - G0[(size_t)j * m + i]));
      }
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < k; ++j) {
        cd u = 0;
        for (int p = 0; p < m; ++p) u += std::conj(G[(size_t)i * m + p]) * G[(size_t)j * m + p];
        un = std::max(un, std::abs(u - (i == j ? 1.0 : 0.0)));
      }
    check(e < 1e-13 && un < 1e-13, "thin QR", m, std::max(e, un));
  }
  // harmonic Ritz pairs of an Arnoldi Hessenberg Hbar ((d+1) x d): with f = H_d^-H conj(h) (h the
  // last row of Hbar), every eigenvector y of H_d + f h^T satisfies
  //   Hbar y - theta [y; 0] = (h^T y) [-f; 1],
  // i.e. all harmonic Ritz residuals are parallel to the least-squares residual direction [-f; 1]
  // (Morgan's lemma), which is what lets the deflated restart keep an Arnoldi-like relation
  for (int d : {4, 8, 16}) {
    std::vector<cd> Hb((size_t)(d + 1) * d, 0.0);
    for (int c = 0; c < d; ++c)
      for (int r = 0; r <= std::min(c + 1, d); ++r) Hb[(size_t)c * (d + 1) + r] = cd(nd(rng), nd(rng));
    for (int c = 0; c < d; ++c) Hb[(size_t)c * (d + 1) + c + 1] = std::abs(nd(rng)) + 0.5;  // subdiagonal norms
    std::vector<cd> Hd((size_t)d * d), f(d), h(d);
    for (int c = 0; c < d; ++c) {
      for (int r = 0; r < d; ++r) Hd[(size_t)c * d + r] = Hb[(size_t)c * (d + 1) + r];
      h[c] = Hb[(size_t)c * (d + 1) + d];
      f[c] = std::conj(h[c]);
    }
    lu_solve(d, Hd, f, true);
    std::vector<cd> M = Hd, Y;
    for (int c = 0; c < d; ++c)
      for (int r = 0; r < d; ++r) M[(size_t)c * d + r] += f[r] * h[c];
    schur(d, M, Y);
    sort_smallest(d, M, Y, 1);
    // the first Schur vector is an eigenvector with eigenvalue M(0,0)
    const cd theta = M[0];
    std::vector<cd> res(d + 1);
    cd hy = 0;
    for (int r = 0; r <= d; ++r) {
      cd s = 0;
      for (int c = 0; c < d; ++c) s += Hb[(size_t)c * (d + 1) + r] * Y[c];
      res[r] = s - (r < d ? theta * Y[r] : cd(0.0));
    }
    for (int c = 0; c < d; ++c) hy += h[c] * Y[c];
    double dev = 0, nr = 0;
    for (int r = 0; r <= d; ++r) {
      const cd want = hy * (r < d ? -f[r] : cd(1.0));
      dev = std::max(dev, std::abs(res[r] - want));
      nr = std::max(nr, std::abs(res[r]));
    }
    check(dev < 1e-10 * std::max(1.0, nr), "harmonic Ritz residual || [-f; 1]", d, dev);
  }
  std::printf("%s\n", fails ? "FAILED" : "all ok");
  return fails ? 1 : 0;
}
