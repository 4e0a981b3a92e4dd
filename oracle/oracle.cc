/*
 * CPU oracle for the even-odd Wilson-clover solve -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker, never the product: only the test-suite, the smoke
 * check and the CPU-baseline leg of the benchmark load it.  It is a plain
 * double-precision (and, for the mixed-precision reliable CG, single-precision)
 * restatement of Chroma 3.44's operator and inverters, one lattice site per loop
 * iteration, OpenMP over sites.  Every routine cites the Chroma source it follows
 * (paths relative to the Chroma tree).
 *
 * Chroma itself cannot be built here (configure.ac:511-568 requires QDP++, which
 * is absent), so the pieces of QDP++ that the path uses are restated from their
 * documented meaning:
 *   - shift(x, FORWARD, mu)(site) = x(site + mu), BACKWARD = x(site - mu), periodic;
 *   - spinProjectDir<mu><Minus|Plus> / spinReconstruct... together apply (1 -/+ gamma_mu);
 *   - gamma matrices in the DeGrand-Rossi basis (docs/notes/gamma_conventions.tex:68-81);
 *   - rb[0] = even sites ((x+y+z+t) mod 2 == 0), rb[1] = odd sites;
 *   - spinor element order (spin, colour), colour matrix element (row, col).
 *
 * Canonical host layouts used throughout (also the C-ABI's host layouts):
 *   site index  s = x + Lx*(y + Ly*(z + Lz*t))
 *   gauge       complex u[s][mu][row][col]            (V*4*9 complex)
 *   spinor      complex psi[s][spin][colour]           (V*12 complex)
 *   clover      per site {double diag[2][6]; complex offd[2][15]}  (72 doubles,
 *               Chroma's PrimitiveClovTriang, clover_term_qdp_w.h:19-24)
 */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

using cd = std::complex<double>;
static constexpr int Nc = 3;
static constexpr int Ns = 4;
static constexpr int NSP = Nc * Ns;  // complex components per spinor site

// ---------------------------------------------------------------------------------------------
// Geometry
// ---------------------------------------------------------------------------------------------
struct Geom {
  int L[4];
  long V, Vh;
  std::vector<long> fwd[4], bwd[4];
  std::vector<int> par;
  std::vector<long> sites[2];  // rb[cb] site table, lexicographic order

  explicit Geom(const int* dims) {
    for (int m = 0; m < 4; ++m) L[m] = dims[m];
    V = (long)L[0] * L[1] * L[2] * L[3];
    Vh = V / 2;
    for (int m = 0; m < 4; ++m) { fwd[m].resize(V); bwd[m].resize(V); }
    par.resize(V);
    for (long s = 0; s < V; ++s) {
      int x[4];
      coords(s, x);
      par[s] = (x[0] + x[1] + x[2] + x[3]) & 1;
      sites[par[s]].push_back(s);
      for (int m = 0; m < 4; ++m) {
        int y[4] = {x[0], x[1], x[2], x[3]};
        y[m] = (x[m] + 1) % L[m];
        fwd[m][s] = lin(y);
        y[m] = (x[m] - 1 + L[m]) % L[m];
        bwd[m][s] = lin(y);
      }
    }
  }
  long lin(const int* x) const { return x[0] + (long)L[0] * (x[1] + (long)L[1] * (x[2] + (long)L[2] * x[3])); }
  void coords(long s, int* x) const {
    x[0] = s % L[0]; s /= L[0];
    x[1] = s % L[1]; s /= L[1];
    x[2] = s % L[2]; s /= L[2];
    x[3] = (int)s;
  }
};

// ---------------------------------------------------------------------------------------------
// Gamma matrices, DeGrand-Rossi basis (docs/notes/gamma_conventions.tex:68-81); mu = 0..3 is
// gamma_1..gamma_4 of the note.
// ---------------------------------------------------------------------------------------------
static const cd I1(0.0, 1.0);
static cd GAMMA[4][4][4];
static cd GAMMA5[4][4];
static bool gamma_ready = false;

static void init_gamma() {
  if (gamma_ready) return;
  for (int m = 0; m < 4; ++m)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) GAMMA[m][a][b] = 0.0;
  // gamma_1 = [[0, i sigma_1], [-i sigma_1, 0]]
  GAMMA[0][0][3] = I1;  GAMMA[0][1][2] = I1;  GAMMA[0][2][1] = -I1; GAMMA[0][3][0] = -I1;
  // gamma_2 = [[0, -i sigma_2], [i sigma_2, 0]]
  GAMMA[1][0][3] = -1.0; GAMMA[1][1][2] = 1.0; GAMMA[1][2][1] = 1.0; GAMMA[1][3][0] = -1.0;
  // gamma_3 = [[0, i sigma_3], [-i sigma_3, 0]]
  GAMMA[2][0][2] = I1;  GAMMA[2][1][3] = -I1; GAMMA[2][2][0] = -I1; GAMMA[2][3][1] = I1;
  // gamma_4 = [[0, 1], [1, 0]]
  GAMMA[3][0][2] = 1.0; GAMMA[3][1][3] = 1.0; GAMMA[3][2][0] = 1.0; GAMMA[3][3][1] = 1.0;
  // gamma_5 = gamma_1 gamma_2 gamma_3 gamma_4
  cd t1[4][4], t2[4][4];
  auto mul = [](cd (*a)[4], cd (*b)[4], cd (*c)[4]) {
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        cd s = 0;
        for (int k = 0; k < 4; ++k) s += a[i][k] * b[k][j];
        c[i][j] = s;
      }
  };
  mul(GAMMA[0], GAMMA[1], t1);
  mul(t1, GAMMA[2], t2);
  mul(t2, GAMMA[3], GAMMA5);
  gamma_ready = true;
}

// ---------------------------------------------------------------------------------------------
// Small SU(3) helpers
// ---------------------------------------------------------------------------------------------
struct M3 {
  cd a[3][3];
};
static inline M3 mzero() { M3 r; for (auto& row : r.a) for (auto& e : row) e = 0.0; return r; }
static inline M3 mone() { M3 r = mzero(); r.a[0][0] = r.a[1][1] = r.a[2][2] = 1.0; return r; }
static inline M3 mmul(const M3& x, const M3& y) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j] + x.a[i][2] * y.a[2][j];
  return r;
}
static inline M3 madj(const M3& x) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r.a[i][j] = std::conj(x.a[j][i]);
  return r;
}
static inline M3 madd(const M3& x, const M3& y) { M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] + y.a[i][j]; return r; }
static inline M3 msub(const M3& x, const M3& y) { M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] - y.a[i][j]; return r; }
static inline M3 mscale(const M3& x, cd f) { M3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.a[i][j] = x.a[i][j] * f; return r; }
static inline cd mtrace(const M3& x) { return x.a[0][0] + x.a[1][1] + x.a[2][2]; }
static inline M3 load_m3(const cd* p) { M3 r; for (int i = 0; i < 9; ++i) r.a[i / 3][i % 3] = p[i]; return r; }
static inline void store_m3(cd* p, const M3& m) { for (int i = 0; i < 9; ++i) p[i] = m.a[i / 3][i % 3]; }
static inline double mnorm_inf(const M3& x) {
  double m = 0;
  for (int i = 0; i < 3; ++i) {
    double r = 0;
    for (int j = 0; j < 3; ++j) r += std::abs(x.a[i][j]);
    m = std::max(m, r);
  }
  return m;
}

// exp(A) for a general 3x3 complex matrix: scaling and squaring around a Taylor series.
static M3 mexp_taylor(const M3& A) {
  double n = mnorm_inf(A);
  int sq = 0;
  while (n > 0.25) { n *= 0.5; ++sq; }
  M3 As = mscale(A, std::ldexp(1.0, -sq));
  M3 term = mone(), sum = mone();
  for (int k = 1; k <= 18; ++k) {
    term = mscale(mmul(term, As), 1.0 / k);
    sum = madd(sum, term);
  }
  for (int i = 0; i < sq; ++i) sum = mmul(sum, sum);
  return sum;
}

// Re-unitarisation by rows (Gram-Schmidt of rows 0 and 1, row 2 = conj(row0 x row1)),
// following lib/util/gauge/reunit.cc:205-262.
static M3 reunit_m3(const M3& u) {
  M3 r = u;
  double n0 = 0;
  for (int c = 0; c < 3; ++c) n0 += std::norm(r.a[0][c]);
  n0 = 1.0 / std::sqrt(n0);
  for (int c = 0; c < 3; ++c) r.a[0][c] *= n0;
  cd ip = 0;
  for (int c = 0; c < 3; ++c) ip += std::conj(r.a[0][c]) * r.a[1][c];
  for (int c = 0; c < 3; ++c) r.a[1][c] -= ip * r.a[0][c];
  double n1 = 0;
  for (int c = 0; c < 3; ++c) n1 += std::norm(r.a[1][c]);
  n1 = 1.0 / std::sqrt(n1);
  for (int c = 0; c < 3; ++c) r.a[1][c] *= n1;
  r.a[2][0] = std::conj(r.a[0][1] * r.a[1][2] - r.a[0][2] * r.a[1][1]);
  r.a[2][1] = std::conj(r.a[0][2] * r.a[1][0] - r.a[0][0] * r.a[1][2]);
  r.a[2][2] = std::conj(r.a[0][0] * r.a[1][1] - r.a[0][1] * r.a[1][0]);
  return r;
}

// ---------------------------------------------------------------------------------------------
// Seeded counter-based random numbers (the synthetic-input recipe shared with the product's
// generator; the recipe is the project's own, Chroma's QDP++ RNG cannot be reproduced here).
//   bits(seed, k)  = mix(mix(seed * 0x9E3779B97F4A7C15 + k))
//   uniform(seed,k)= ((bits >> 11) + 0.5) * 2^-53            in (0, 1)
//   normal(seed,k) = sqrt(-2 ln uniform(seed,2k)) * cos(2 pi uniform(seed,2k+1))
// ---------------------------------------------------------------------------------------------
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static inline uint64_t rbits(uint64_t seed, uint64_t k) { return mix64(mix64(seed * 0x9E3779B97F4A7C15ULL + k)); }
static inline double runiform(uint64_t seed, uint64_t k) { return ((double)(rbits(seed, k) >> 11) + 0.5) * 0x1.0p-53; }
static inline double rnormal(uint64_t seed, uint64_t k) {
  double u1 = runiform(seed, 2 * k), u2 = runiform(seed, 2 * k + 1);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586476925286766559 * u2);
}

// ---------------------------------------------------------------------------------------------
// Stout smearing (lib/util/gauge/stout_utils.cc:105-180 getQsandCs, :936-966 smear_links)
// with exp(iQ) by the Cayley-Hamilton method of Morningstar & Peardon, PRD 69 (2004) 054501,
// as in stout_utils.cc:415-700 (a Taylor series replaces its small-c1 polynomial branch).
// ---------------------------------------------------------------------------------------------
static M3 exp_iQ(const M3& Q) {
  M3 QQ = mmul(Q, Q);
  double c0 = std::real(mtrace(mmul(QQ, Q))) / 3.0;
  double c1 = std::real(mtrace(QQ)) / 2.0;
  if (c1 < 4.0e-3) return mexp_taylor(mscale(Q, I1));
  bool neg = c0 < 0;
  double c0a = std::fabs(c0);
  double c0max = 2.0 * std::pow(c1 / 3.0, 1.5);
  double ratio = std::min(1.0, c0a / c0max);
  double theta = std::acos(ratio);
  double u = std::sqrt(c1 / 3.0) * std::cos(theta / 3.0);
  double w = std::sqrt(c1) * std::sin(theta / 3.0);
  double u2 = u * u, w2 = w * w;
  double xi0 = (std::fabs(w) < 0.05) ? 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0)) : std::sin(w) / w;
  double cw = std::cos(w);
  cd e2iu = std::exp(cd(0, 2 * u)), emiu = std::exp(cd(0, -u));
  cd h0 = (u2 - w2) * e2iu + emiu * (8.0 * u2 * cw + cd(0, 2.0 * u * (3.0 * u2 + w2)) * xi0);
  cd h1 = 2.0 * u * e2iu - emiu * (2.0 * u * cw - cd(0, (3.0 * u2 - w2)) * xi0);
  cd h2 = e2iu - emiu * (cw + cd(0, 3.0 * u) * xi0);
  double den = 1.0 / (9.0 * u2 - w2);
  cd f0 = h0 * den, f1 = h1 * den, f2 = h2 * den;
  if (neg) { f0 = std::conj(f0); f1 = -std::conj(f1); f2 = std::conj(f2); }
  M3 r = mone();
  r = mscale(r, f0);
  r = madd(r, mscale(Q, f1));
  r = madd(r, mscale(QQ, f2));
  return r;
}

static inline M3 link(const std::vector<cd>& u, long s, int mu) { return load_m3(&u[(s * 4 + mu) * 9]); }

static void stout_step(const Geom& g, const std::vector<cd>& cur, std::vector<cd>& nxt, double rho,
                       const int* smear_dir) {
  nxt.resize(cur.size());
#pragma omp parallel for schedule(static)
  for (long s = 0; s < g.V; ++s) {
    for (int mu = 0; mu < 4; ++mu) {
      M3 U = link(cur, s, mu);
      if (!smear_dir[mu]) { store_m3(&nxt[(s * 4 + mu) * 9], U); continue; }
      M3 C = mzero();
      for (int nu = 0; nu < 4; ++nu) {
        if (nu == mu || !smear_dir[nu]) continue;
        long sp_mu = g.fwd[mu][s], sp_nu = g.fwd[nu][s], sm_nu = g.bwd[nu][s];
        long sm_nu_p_mu = g.fwd[mu][sm_nu];
        // forward staple U_nu(x) U_mu(x+nu) U_nu^dag(x+mu)
        M3 st = mmul(mmul(link(cur, s, nu), link(cur, sp_nu, mu)), madj(link(cur, sp_mu, nu)));
        // backward staple U_nu^dag(x-nu) U_mu(x-nu) U_nu(x-nu+mu)
        st = madd(st, mmul(mmul(madj(link(cur, sm_nu, nu)), link(cur, sm_nu, mu)), link(cur, sm_nu_p_mu, nu)));
        C = madd(C, mscale(st, rho));
      }
      M3 Om = mmul(C, madj(U));
      M3 t2 = msub(madj(Om), Om);
      cd tr = mtrace(t2) / 3.0;
      for (int i = 0; i < 3; ++i) t2.a[i][i] -= tr;
      M3 Q = mscale(t2, cd(0, 0.5));
      store_m3(&nxt[(s * 4 + mu) * 9], mmul(exp_iQ(Q), U));
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Clover term: mesField (lib/meas/glue/mesfield.cc:30-78), makeClov
// (lib/actions/ferm/linop/clover_term_qdp_w.h:244-294, 398-553), LDL^dag inverse (:608-846),
// apply (:1553-1620, 2138-2160).
// ---------------------------------------------------------------------------------------------
template <typename R>
struct CloverSite {
  R diag[2][6];
  std::complex<R> offd[2][15];
};
static_assert(sizeof(CloverSite<double>) == 72 * sizeof(double), "packed clover is 72 reals");

// F(mu,nu) = (1/8) [Q - Q^dag], Q = sum of the four leaves, for the pairs
// (0,1),(0,2),(0,3),(1,2),(1,3),(2,3) in that order.
static void mesfield(const Geom& g, const std::vector<cd>& u, std::vector<M3>& f) {
  f.resize(6 * g.V);
#pragma omp parallel for schedule(static)
  for (long s = 0; s < g.V; ++s) {
    int off = 0;
    for (int mu = 0; mu < 3; ++mu)
      for (int nu = mu + 1; nu < 4; ++nu, ++off) {
        long xpm = g.fwd[mu][s], xpn = g.fwd[nu][s], xmm = g.bwd[mu][s], xmn = g.bwd[nu][s];
        long xmm_pn = g.fwd[nu][xmm], xmm_mn = g.bwd[nu][xmm], xmn_pm = g.fwd[mu][xmn];
        // U_1 = u(x,mu) u(x+mu,nu) u^dag(x+nu,mu) u^dag(x,nu)
        M3 q = mmul(mmul(mmul(link(u, s, mu), link(u, xpm, nu)), madj(link(u, xpn, mu))), madj(link(u, s, nu)));
        // U_2 = u(x,nu) u^dag(x-mu+nu,mu) u^dag(x-mu,nu) u(x-mu,mu)
        q = madd(q, mmul(mmul(mmul(link(u, s, nu), madj(link(u, xmm_pn, mu))), madj(link(u, xmm, nu))), link(u, xmm, mu)));
        // U_3 = u^dag(x-mu,mu) u^dag(x-mu-nu,nu) u(x-mu-nu,mu) u(x-nu,nu)
        q = madd(q, mmul(mmul(mmul(madj(link(u, xmm, mu)), madj(link(u, xmm_mn, nu))), link(u, xmm_mn, mu)), link(u, xmn, nu)));
        // U_4 = u^dag(x-nu,nu) u(x-nu,mu) u(x-nu+mu,nu) u^dag(x,mu)
        q = madd(q, mmul(mmul(mmul(madj(link(u, xmn, nu)), link(u, xmn, mu)), link(u, xmn_pm, nu)), madj(link(u, s, mu))));
        f[6 * s + off] = mscale(msub(q, madj(q)), 0.125);
      }
  }
}

struct CloverParams {
  double mass;
  double clov_coeff_r, clov_coeff_t;
  int aniso;       // anisoParam.anisoP
  double xi_0, nu; // anisoParam.xi_0, anisoParam.nu
  int t_dir;       // anisoParam.t_dir
};

// makeClov site body (clover_term_qdp_w.h:398-553), with f_k pre-multiplied by
// getCloverCoeff (clover_term_qdp_w.h:513-519, 1527-1549) and the 1/2 of create (:263-267).
static void make_clover(const Geom& g, const std::vector<cd>& u, const CloverParams& p,
                        std::vector<CloverSite<double>>& tri) {
  std::vector<M3> f;
  mesfield(g, u, f);
  double ffR = p.aniso ? 1.0 / p.xi_0 : 1.0;
  double cR = p.clov_coeff_r * 0.5 * ffR;
  double cT = p.clov_coeff_t * 0.5;
  double ffm = p.aniso ? p.nu / p.xi_0 : 1.0;
  double diag_mass = 1.0 + (4 - 1) * ffm + p.mass;
  const int pairs[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  double coef[6];
  for (int k = 0; k < 6; ++k) {
    bool t = p.aniso && (pairs[k][0] == p.t_dir || pairs[k][1] == p.t_dir);
    coef[k] = p.aniso ? (t ? cT : cR) : cR;
  }
  tri.resize(g.V);
#pragma omp parallel for schedule(static)
  for (long s = 0; s < g.V; ++s) {
    M3 F[6];
    for (int k = 0; k < 6; ++k) F[k] = mscale(f[6 * s + k], coef[k]);
    CloverSite<double>& T = tri[s];
    for (int b = 0; b < 2; ++b)
      for (int i = 0; i < 6; ++i) T.diag[b][i] = diag_mass;
    for (int i = 0; i < Nc; ++i) {
      double r0 = std::imag(F[5].a[i][i] - F[0].a[i][i]);
      T.diag[0][i] += r0;
      T.diag[0][i + Nc] -= r0;
      double r1 = std::imag(F[5].a[i][i] + F[0].a[i][i]);
      T.diag[1][i] -= r1;
      T.diag[1][i + Nc] += r1;
    }
    for (int i = 1; i < Nc; ++i)
      for (int j = 0; j < i; ++j) {
        int eij = i * (i - 1) / 2 + j;
        int etmp = (i + Nc) * (i + Nc - 1) / 2 + j + Nc;
        T.offd[0][eij] = I1 * (F[0].a[i][j] - F[5].a[i][j]);
        T.offd[0][etmp] = -T.offd[0][eij];
        T.offd[1][eij] = I1 * (F[5].a[i][j] + F[0].a[i][j]);
        T.offd[1][etmp] = -T.offd[1][eij];
      }
    for (int i = 0; i < Nc; ++i)
      for (int j = 0; j < Nc; ++j) {
        int eij = (i + Nc) * (i + Nc - 1) / 2 + j;
        cd Em = I1 * F[2].a[i][j] + F[4].a[i][j];
        cd Bm = I1 * F[3].a[i][j] - F[1].a[i][j];
        T.offd[0][eij] = Bm - Em;
        T.offd[1][eij] = Em + Bm;
      }
  }
}

// LDL^dag factorisation and inverse of each 6x6 block (clover_term_qdp_w.h:608-846).
// Returns sum over the sites of parity cb of log|d_i|, counts negative d_i.
template <typename R>
static void ldl_invert_site(CloverSite<R>& T, double& logdet, int& nneg) {
  const int N = 6;
  for (int b = 0; b < 2; ++b) {
    double d[N];
    cd o[15], v[N];
    for (int i = 0; i < N; ++i) d[i] = T.diag[b][i];
    for (int i = 0; i < 15; ++i) o[i] = cd(T.offd[b][i]);
    for (int j = 0; j < N; ++j) {
      for (int i = 0; i < j; ++i) v[i] = d[i] * std::conj(o[j * (j - 1) / 2 + i]);
      v[j] = d[j];
      for (int k = 0; k < j; ++k) v[j] -= o[j * (j - 1) / 2 + k] * v[k];
      d[j] = std::real(v[j]);
      for (int k = j + 1; k < N; ++k) {
        int ekj = k * (k - 1) / 2 + j;
        for (int l = 0; l < j; ++l) o[ekj] -= o[k * (k - 1) / 2 + l] * v[l];
        o[ekj] /= v[j];
      }
    }
    double dg[N];
    for (int i = 0; i < N; ++i) {
      dg[i] = 1.0 / d[i];
      logdet += std::log(std::fabs(d[i]));
      if (d[i] < 0) ++nneg;
    }
    double inv_d[N];
    cd inv_o[15];
    for (int i = 0; i < 15; ++i) inv_o[i] = o[i];
    for (int i = 0; i < N; ++i) inv_d[i] = d[i];
    for (int k = 0; k < N; ++k) {
      for (int i = 0; i < k; ++i) v[i] = 0;
      v[k] = dg[k];
      for (int i = k + 1; i < N; ++i) {
        v[i] = 0;
        for (int j = k; j < i; ++j) v[i] -= o[i * (i - 1) / 2 + j] * d[j] * v[j];
        v[i] *= dg[i];
      }
      for (int i = N - 2; i >= k; --i)
        for (int j = i + 1; j < N; ++j) v[i] -= std::conj(o[j * (j - 1) / 2 + i]) * v[j];
      inv_d[k] = std::real(v[k]);
      for (int i = k + 1; i < N; ++i) inv_o[i * (i - 1) / 2 + k] = v[i];
    }
    for (int i = 0; i < N; ++i) T.diag[b][i] = (R)inv_d[i];
    for (int i = 0; i < 15; ++i) T.offd[b][i] = std::complex<R>((R)inv_o[i].real(), (R)inv_o[i].imag());
  }
}

// ---------------------------------------------------------------------------------------------
// Operator in precision R: links with the anisotropy coefficients folded in (lwldslash_w.h:182-212),
// the clover term on both parities and its inverse on the even parity
// (eoprec_clover_linop_w.cc:19-39).
// ---------------------------------------------------------------------------------------------
template <typename R>
struct Op {
  const Geom* g;
  std::vector<std::complex<R>> u;     // dslash links
  std::vector<CloverSite<R>> clov;     // A on all sites
  std::vector<CloverSite<R>> invclov;  // A^-1 on all sites (the odd ones serve the symmetric operator)
  bool twisted = false;
  R twisted_m = 0;
  double logdet_even = 0;   // cholesDet(0)
  double logdet_odd = 0;    // cholesDet(1), the symmetric operator's logDetOddOddLinOp
  int nneg = 0;
};

using spin_t = std::complex<double>;

// Wilson hopping term D' on the sites of parity cb (lwldslash_w.h:16-44, 226-303).
template <typename R>
static void dslash(const Op<R>& op, std::complex<R>* chi, const std::complex<R>* psi, int isign, int cb) {
  const Geom& g = *op.g;
  const auto& sites = g.sites[cb];
  const long n = (long)sites.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    long s = sites[i];
    std::complex<R> acc[NSP];
    for (auto& a : acc) a = 0;
    for (int mu = 0; mu < 4; ++mu) {
      for (int dir = 0; dir < 2; ++dir) {
        // dir 0: U_mu(x) (1 - isign gamma_mu) psi(x+mu)
        // dir 1: U_mu^dag(x-mu) (1 + isign gamma_mu) psi(x-mu)
        long nb = dir == 0 ? g.fwd[mu][s] : g.bwd[mu][s];
        R sg = (R)(dir == 0 ? -isign : isign);
        const std::complex<R>* p = psi + nb * NSP;
        std::complex<R> t[NSP];
        for (int a = 0; a < Ns; ++a)
          for (int c = 0; c < Nc; ++c) {
            std::complex<R> v = p[a * Nc + c];
            for (int b = 0; b < Ns; ++b) {
              cd gm = GAMMA[mu][a][b];
              if (gm != 0.0) v += sg * std::complex<R>((R)gm.real(), (R)gm.imag()) * p[b * Nc + c];
            }
            t[a * Nc + c] = v;
          }
        long ls = dir == 0 ? s : nb;
        const std::complex<R>* U = &op.u[(ls * 4 + mu) * 9];
        for (int a = 0; a < Ns; ++a)
          for (int r = 0; r < Nc; ++r) {
            std::complex<R> v = 0;
            for (int c = 0; c < Nc; ++c)
              v += (dir == 0 ? U[r * 3 + c] : std::conj(U[c * 3 + r])) * t[a * Nc + c];
            acc[a * Nc + r] += v;
          }
      }
    }
    for (int k = 0; k < NSP; ++k) chi[s * NSP + k] = acc[k];
  }
}

// chi = T psi on parity cb for packed Hermitian blocks T (clover_term_qdp_w.h:1553-1620).
template <typename R>
static void clover_apply(const Op<R>& op, const std::vector<CloverSite<R>>& tri, std::complex<R>* chi,
                         const std::complex<R>* psi, int cb) {
  const Geom& g = *op.g;
  const auto& sites = g.sites[cb];
  const long n = (long)sites.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    long s = sites[i];
    const CloverSite<R>& T = tri[s];
    const std::complex<R>* p = psi + s * NSP;
    std::complex<R>* c = chi + s * NSP;
    for (int b = 0; b < 2; ++b) {
      for (int k = 0; k < 6; ++k) c[6 * b + k] = T.diag[b][k] * p[6 * b + k];
      int kij = 0;
      for (int a = 0; a < 6; ++a)
        for (int j = 0; j < a; ++j, ++kij) {
          c[6 * b + a] += T.offd[b][kij] * p[6 * b + j];
          c[6 * b + j] += std::conj(T.offd[b][kij]) * p[6 * b + a];
        }
    }
  }
}

// Even-odd preconditioned operator  chi_o = A_oo psi_o - 1/4 D_oe A_ee^-1 D_eo psi_o
// (+ isign * i mu gamma_5 psi_o when twisted), eoprec_clover_linop_w.cc:142-187.
template <typename R>
static void eo_op(const Op<R>& op, std::complex<R>* chi, const std::complex<R>* psi, int isign) {
  const Geom& g = *op.g;
  std::vector<std::complex<R>> t1(g.V * NSP), t2(g.V * NSP);
  dslash(op, t1.data(), psi, isign, 0);
  clover_apply(op, op.invclov, t2.data(), t1.data(), 0);
  dslash(op, t1.data(), t2.data(), isign, 1);
  clover_apply(op, op.clov, chi, psi, 1);
  const auto& sites = g.sites[1];
  const long n = (long)sites.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    long s = sites[i];
    for (int k = 0; k < NSP; ++k) chi[s * NSP + k] += (R)(-0.25) * t1[s * NSP + k];
    if (op.twisted) {
      // gamma_5 = diag(1,1,-1,-1) in this basis; verified against GAMMA5 at init
      for (int a = 0; a < Ns; ++a) {
        R g5 = (R)GAMMA5[a][a].real();
        for (int c = 0; c < Nc; ++c) {
          std::complex<R> v = psi[s * NSP + a * Nc + c] * std::complex<R>(0, g5 * op.twisted_m);
          chi[s * NSP + a * Nc + c] += (R)isign * v;
        }
      }
    }
  }
}

// Symmetric even-odd preconditioned operator (seoprec_clover_linop_w.cc:145-187):
//   PLUS:  chi_o = psi_o - 1/4 A_oo^-1 D_oe A_ee^-1 D_eo psi_o
//   MINUS: chi_o = psi_o - 1/4 D_oe^dag A_ee^-1 D_eo^dag A_oo^-1 psi_o   (its adjoint)
// (+ isign * i mu gamma_5 psi_o when twisted).  A_oo^-1 M~ = this operator for PLUS.
template <typename R>
static void sym_op(const Op<R>& op, std::complex<R>* chi, const std::complex<R>* psi, int isign) {
  const Geom& g = *op.g;
  std::vector<std::complex<R>> t1(g.V * NSP), t2(g.V * NSP);
  if (isign > 0) {
    dslash(op, t1.data(), psi, isign, 0);
    clover_apply(op, op.invclov, t2.data(), t1.data(), 0);
    dslash(op, t1.data(), t2.data(), isign, 1);
    clover_apply(op, op.invclov, t2.data(), t1.data(), 1);
  } else {
    clover_apply(op, op.invclov, t1.data(), psi, 1);
    dslash(op, t2.data(), t1.data(), isign, 0);
    clover_apply(op, op.invclov, t1.data(), t2.data(), 0);
    dslash(op, t2.data(), t1.data(), isign, 1);
  }
  const auto& sites = g.sites[1];
  const long n = (long)sites.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    long s = sites[i];
    for (int k = 0; k < NSP; ++k) chi[s * NSP + k] = psi[s * NSP + k] + (R)(-0.25) * t2[s * NSP + k];
    if (op.twisted) {
      for (int a = 0; a < Ns; ++a) {
        R g5 = (R)GAMMA5[a][a].real();
        for (int c = 0; c < Nc; ++c) {
          std::complex<R> v = psi[s * NSP + a * Nc + c] * std::complex<R>(0, g5 * op.twisted_m);
          chi[s * NSP + a * Nc + c] += (R)isign * v;
        }
      }
    }
  }
}

// Unpreconditioned operator (lib/eoprec_linop.h:147-165):
//   chi_e = A_ee psi_e - 1/2 D_eo psi_o,   chi_o = -1/2 D_oe psi_e + A_oo psi_o
template <typename R>
static void unprec_op(const Op<R>& op, std::complex<R>* chi, const std::complex<R>* psi, int isign) {
  const Geom& g = *op.g;
  std::vector<std::complex<R>> t1(g.V * NSP), t2(g.V * NSP);
  for (int cb = 0; cb < 2; ++cb) {
    clover_apply(op, op.clov, t1.data(), psi, cb);
    dslash(op, t2.data(), psi, isign, cb);
    for (long s : g.sites[cb])
      for (int k = 0; k < NSP; ++k) chi[s * NSP + k] = t1[s * NSP + k] + (R)(-0.5) * t2[s * NSP + k];
  }
}

// ---------------------------------------------------------------------------------------------
// BLAS-1 on a parity subset, FP64 accumulation
// ---------------------------------------------------------------------------------------------
template <typename R>
static double norm2_cb(const Geom& g, const std::complex<R>* x, int cb) {
  const auto& sites = g.sites[cb];
  const long n = (long)sites.size();
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long i = 0; i < n; ++i) {
    const std::complex<R>* p = x + sites[i] * NSP;
    for (int k = 0; k < NSP; ++k) s += (double)std::norm(p[k]);
  }
  return s;
}

static cd inner_cb(const Geom& g, const cd* x, const cd* y, int cb) {
  const auto& sites = g.sites[cb];
  const long n = (long)sites.size();
  double re = 0, im = 0;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
  for (long i = 0; i < n; ++i) {
    long s = sites[i];
    for (int k = 0; k < NSP; ++k) {
      cd v = std::conj(x[s * NSP + k]) * y[s * NSP + k];
      re += v.real();
      im += v.imag();
    }
  }
  return cd(re, im);
}

// y[cb] = a*x + b*y
template <typename R, typename S>
static void axpby_cb(const Geom& g, S a, const std::complex<R>* x, S b, std::complex<R>* y, int cb) {
  const auto& sites = g.sites[cb];
  const long n = (long)sites.size();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) {
    long s = sites[i];
    for (int k = 0; k < NSP; ++k) y[s * NSP + k] = a * x[s * NSP + k] + b * y[s * NSP + k];
  }
}

struct SolveResult {
  int n_count;
  double resid;       // absolute true residual |chi - M psi| on rb[1]
  double rel_resid;   // resid / |chi|
};

// InvCG2 (lib/actions/ferm/invert/invcg2.cc:70-232) on M^dag M, restricted to rb[1].
static SolveResult invcg2(const Op<double>& M, const cd* chi, cd* psi, double RsdCG, int MaxCG) {
  const Geom& g = *M.g;
  const long N = g.V * NSP;
  std::vector<cd> mp(N), mmp(N), p(N), r(N);
  SolveResult res{0, 0, 0};
  double chi_sq = norm2_cb(g, chi, 1);
  double rsd_sq = RsdCG * RsdCG * chi_sq;
  eo_op(M, mp.data(), psi, +1);
  eo_op(M, mmp.data(), mp.data(), -1);
  for (long s : g.sites[1])
    for (int k = 0; k < NSP; ++k) r[s * NSP + k] = chi[s * NSP + k] - mmp[s * NSP + k];
  double cp = norm2_cb(g, r.data(), 1);
  for (long s : g.sites[1])
    for (int k = 0; k < NSP; ++k) p[s * NSP + k] = r[s * NSP + k];
  if (cp <= rsd_sq) { res.n_count = 0; res.resid = std::sqrt(cp); return res; }
  for (int k = 1; k <= MaxCG; ++k) {
    double c = cp;
    eo_op(M, mp.data(), p.data(), +1);
    double d = norm2_cb(g, mp.data(), 1);
    eo_op(M, mmp.data(), mp.data(), -1);
    double a = c / d;
    axpby_cb<double, double>(g, -a, mmp.data(), 1.0, r.data(), 1);
    cp = norm2_cb(g, r.data(), 1);
    axpby_cb<double, double>(g, a, p.data(), 1.0, psi, 1);
    if (cp <= rsd_sq) {
      res.n_count = k;
      res.resid = std::sqrt(cp);
      return res;
    }
    double b = cp / c;
    axpby_cb<double, double>(g, 1.0, r.data(), b, p.data(), 1);
  }
  res.n_count = MaxCG;
  res.resid = std::sqrt(cp);
  return res;
}

static double true_resid_linop(const Op<double>& M, const cd* chi, const cd* psi) {
  const Geom& g = *M.g;
  std::vector<cd> t(g.V * NSP), r(g.V * NSP);
  eo_op(M, t.data(), psi, +1);
  for (long s : g.sites[1])
    for (int k = 0; k < NSP; ++k) r[s * NSP + k] = chi[s * NSP + k] - t[s * NSP + k];
  return std::sqrt(norm2_cb(g, r.data(), 1));
}

// LinOpSysSolverCG (lib/actions/ferm/invert/syssolver_linop_cg.h:57-96): chi' = M^dag chi,
// InvCG2 on M^dag M, then the true residual of M psi = chi on rb[1].
static SolveResult linop_cg(const Op<double>& M, const cd* chi, cd* psi, double rsd, int maxit) {
  const Geom& g = *M.g;
  std::vector<cd> chit(g.V * NSP);
  eo_op(M, chit.data(), chi, -1);
  SolveResult res = invcg2(M, chit.data(), psi, rsd, maxit);
  res.resid = true_resid_linop(M, chi, psi);
  res.rel_resid = res.resid / std::sqrt(norm2_cb(g, chi, 1));
  return res;
}

// RelInvCG_a (lib/actions/ferm/invert/reliable_cg.cc:10-188): CG on M^dag M with the iterated
// vectors and the operator in single precision, reliable updates of the residual in double.
static SolveResult reliable_cg(const Op<double>& A, const Op<float>& AF, const cd* chi, cd* psi, double RsdCG,
                               double Delta, int MaxCG) {
  const Geom& g = *A.g;
  const long N = g.V * NSP;
  using cf = std::complex<float>;
  std::vector<cd> b(N), r_dble(N), x_dble(N), t1(N), t2(N);
  std::vector<cf> r(N), x(N), p(N), mp(N), mmp(N);
  SolveResult ret{0, 0, 0};
  const auto& odd = g.sites[1];
  for (long s : odd) for (int k = 0; k < NSP; ++k) b[s * NSP + k] = chi[s * NSP + k];
  double chi_norm = norm2_cb(g, chi, 1);
  double rsd_sq = RsdCG * RsdCG * chi_norm;
  eo_op(A, t1.data(), psi, +1);
  eo_op(A, t2.data(), t1.data(), -1);
  for (long s : odd) for (int k = 0; k < NSP; ++k) {
    long i = s * NSP + k;
    b[i] -= t2[i];
    r[i] = cf((float)b[i].real(), (float)b[i].imag());
    x[i] = 0;
  }
  double r_sq = norm2_cb(g, r.data(), 1);
  double rNorm = std::sqrt(r_sq), r0Norm = rNorm, maxrx = rNorm, maxrr = rNorm;
  double c = 0, d, a;
  bool convP = false;
  int k;
  for (k = 0; k < MaxCG && !convP; ++k) {
    if (k == 0) {
      for (long s : odd) for (int q = 0; q < NSP; ++q) p[s * NSP + q] = r[s * NSP + q];
    } else {
      float br = (float)(r_sq / c);
      axpby_cb<float, float>(g, 1.0f, r.data(), br, p.data(), 1);
    }
    c = r_sq;
    eo_op(AF, mp.data(), p.data(), +1);
    d = norm2_cb(g, mp.data(), 1);
    eo_op(AF, mmp.data(), mp.data(), -1);
    a = c / d;
    float ar = (float)a;
    axpby_cb<float, float>(g, ar, p.data(), 1.0f, x.data(), 1);
    axpby_cb<float, float>(g, -ar, mmp.data(), 1.0f, r.data(), 1);
    r_sq = norm2_cb(g, r.data(), 1);
    rNorm = std::sqrt(r_sq);
    if (rNorm > maxrx) maxrx = rNorm;
    if (rNorm > maxrr) maxrr = rNorm;
    bool updateX = (rNorm < Delta * r0Norm && r0Norm <= maxrx);
    bool updateR = (rNorm < Delta * maxrr && r0Norm <= maxrr) || updateX;
    if (updateR) {
      for (long s : odd) for (int q = 0; q < NSP; ++q) { long i = s * NSP + q; x_dble[i] = cd(x[i].real(), x[i].imag()); }
      eo_op(A, t1.data(), x_dble.data(), +1);
      eo_op(A, t2.data(), t1.data(), -1);
      for (long s : odd) for (int q = 0; q < NSP; ++q) {
        long i = s * NSP + q;
        r_dble[i] = b[i] - t2[i];
        r[i] = cf((float)r_dble[i].real(), (float)r_dble[i].imag());
      }
      r_sq = norm2_cb(g, r_dble.data(), 1);
      rNorm = std::sqrt(r_sq);
      maxrr = rNorm;
      if (updateX) {
        for (long s : odd) for (int q = 0; q < NSP; ++q) {
          long i = s * NSP + q;
          psi[i] += x_dble[i];
          x[i] = 0;
          b[i] = r_dble[i];
        }
        r0Norm = rNorm;
        maxrx = rNorm;
      }
    }
    if (r_sq < rsd_sq) {
      for (long s : odd) for (int q = 0; q < NSP; ++q) { long i = s * NSP + q; psi[i] += cd(x[i].real(), x[i].imag()); }
      ret.resid = rNorm;
      ret.n_count = k;
      convP = true;
    }
  }
  if (!convP) ret.n_count = -1;  // Chroma aborts here (reliable_cg.cc:180-183); report it instead
  return ret;
}

// ---------------------------------------------------------------------------------------------
// InvBiCGStab_a (lib/actions/ferm/invert/invbicgstab.cc:12-200) on M itself, restricted to rb[1]:
// r = r0 = chi - M psi, p = v = 0, rho_prev = alpha = omega = 1; per iteration
// rho = <r0|r>, beta = (rho/rho_prev)(alpha/omega), p = r + beta (p - omega v), v = M p,
// alpha = rho/<r0|v>, s = r - alpha v, t = M s, omega = <t|s>/|t|^2, psi += alpha p + omega s,
// r = s - omega t; stop when |r|^2 < RsdBiCGStab^2 |chi|^2 (or rho = 0: breakdown, n_count = -1).
static SolveResult invbicgstab(const Op<double>& M, const cd* chi, cd* psi, double rsd, int maxit) {
  const Geom& g = *M.g;
  const long N = g.V * NSP;
  const auto& odd = g.sites[1];
  std::vector<cd> r(N), r0(N), p(N), v(N), t(N);
  SolveResult res{maxit, 0, 0};
  const double chi_sq = norm2_cb(g, chi, 1);
  const double rsd_sq = rsd * rsd * chi_sq;
  eo_op(M, r0.data(), psi, +1);
  for (long s : odd)
    for (int k = 0; k < NSP; ++k) {
      const long i = s * NSP + k;
      r[i] = r0[i] = chi[i] - r0[i];
    }
  cd rho_prev(1.0), alpha(1.0), omega(1.0);
  double rn = norm2_cb(g, r.data(), 1);
  for (int k = 1; k <= maxit; ++k) {
    const cd rho = inner_cb(g, r0.data(), r.data(), 1);
    if (rho == cd(0.0)) {
      res.n_count = -1;
      break;
    }
    const cd beta = (rho / rho_prev) * (alpha / omega);
    for (long s : odd)
      for (int q = 0; q < NSP; ++q) {
        const long i = s * NSP + q;
        p[i] = r[i] + beta * (p[i] - omega * v[i]);
      }
    eo_op(M, v.data(), p.data(), +1);
    alpha = rho / inner_cb(g, r0.data(), v.data(), 1);
    rho_prev = rho;
    axpby_cb<double, cd>(g, -alpha, v.data(), cd(1.0), r.data(), 1);  // r now holds s
    eo_op(M, t.data(), r.data(), +1);
    omega = inner_cb(g, t.data(), r.data(), 1) / norm2_cb(g, t.data(), 1);
    for (long s : odd)
      for (int q = 0; q < NSP; ++q) {
        const long i = s * NSP + q;
        psi[i] += omega * r[i] + alpha * p[i];
        r[i] -= omega * t[i];
      }
    rn = norm2_cb(g, r.data(), 1);
    if (rn < rsd_sq) {
      res.n_count = k;
      break;
    }
  }
  res.resid = true_resid_linop(M, chi, psi);
  res.rel_resid = res.resid / std::sqrt(chi_sq);
  return res;
}

// RelInvBiCGStab_a (lib/actions/ferm/invert/reliable_bicgstab.cc:18-277): BiCGStab on M with the
// iterated vectors (r, r0, x, p, v, t) and the operator in single precision, inner products summed
// in double, and reliable updates in double: whenever |r| fell below Delta times its largest value
// since the last update, r = b - M x_dble; when it fell below Delta |r| at the last x update, x
// is also folded into psi and the system restarted from the new residual (b = r_dble, x = 0).
static SolveResult rel_bicgstab(const Op<double>& A, const Op<float>& AF, const cd* chi, cd* psi, double rsd,
                                double Delta, int maxit) {
  const Geom& g = *A.g;
  const long N = g.V * NSP;
  const auto& odd = g.sites[1];
  using cf = std::complex<float>;
  std::vector<cd> b(N), tmp(N), r_dble(N), x_dble(N);
  std::vector<cf> r(N), r0(N), x(N), p(N), v(N), t(N);
  auto dot = [&](const std::vector<cf>& a, const std::vector<cf>& c) {  // <a|c> on rb[1], double sums
    double re = 0, im = 0;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
    for (long i = 0; i < (long)odd.size(); ++i)
      for (int k = 0; k < NSP; ++k) {
        const long q = odd[i] * NSP + k;
        const cd u = std::conj(cd(a[q])) * cd(c[q]);
        re += u.real();
        im += u.imag();
      }
    return cd(re, im);
  };
  SolveResult res{maxit, 0, 0};
  const double rsd_sq = rsd * rsd * norm2_cb(g, chi, 1);
  eo_op(A, tmp.data(), psi, +1);
  for (long s : odd)
    for (int k = 0; k < NSP; ++k) {
      const long q = s * NSP + k;
      b[q] = chi[q] - tmp[q];
      r[q] = r0[q] = cf((float)b[q].real(), (float)b[q].imag());
    }
  double r_sq = norm2_cb(g, b.data(), 1);
  double rNorm = std::sqrt(r_sq), r0Norm = rNorm, maxrx = rNorm, maxrr = rNorm;
  cd rho = r_sq, rho_prev = 1.0, alpha = 1.0, omega = 1.0;
  int k;
  for (k = 0; k < maxit; ++k) {
    if (k == 0) {
      p = r;
    } else {
      const cf beta((rho / rho_prev) * (alpha / omega)), om(omega);
      for (long s : odd)
        for (int q = 0; q < NSP; ++q) {
          const long i = s * NSP + q;
          p[i] = r[i] + beta * (p[i] - om * v[i]);
        }
    }
    eo_op(AF, v.data(), p.data(), +1);
    const cd r0v = dot(r0, v);
    if (r0v == cd(0.0)) {
      res.n_count = -1;  // breakdown: Chroma aborts (reliable_bicgstab.cc:146-149)
      break;
    }
    alpha = rho / r0v;
    rho_prev = rho;
    const cf al(alpha);
    for (long s : odd)
      for (int q = 0; q < NSP; ++q) r[s * NSP + q] -= al * v[s * NSP + q];  // r now holds s
    eo_op(AF, t.data(), r.data(), +1);
    double t_norm = 0;
    for (long s : odd)
      for (int q = 0; q < NSP; ++q) t_norm += (double)std::norm(t[s * NSP + q]);
    omega = dot(t, r) / t_norm;
    const cf om(omega);
    for (long s : odd)
      for (int q = 0; q < NSP; ++q) {
        const long i = s * NSP + q;
        x[i] += om * r[i] + al * p[i];
        r[i] -= om * t[i];
      }
    r_sq = 0;
    for (long s : odd)
      for (int q = 0; q < NSP; ++q) r_sq += (double)std::norm(r[s * NSP + q]);
    rho = dot(r0, r);
    rNorm = std::sqrt(r_sq);
    maxrx = std::max(maxrx, rNorm);
    maxrr = std::max(maxrr, rNorm);
    const bool updateX = rNorm < Delta * r0Norm && r0Norm <= maxrx;
    const bool updateR = (rNorm < Delta * maxrr && r0Norm <= maxrr) || updateX;
    if (updateR) {
      for (long s : odd)
        for (int q = 0; q < NSP; ++q) x_dble[s * NSP + q] = cd(x[s * NSP + q]);
      eo_op(A, tmp.data(), x_dble.data(), +1);
      for (long s : odd)
        for (int q = 0; q < NSP; ++q) {
          const long i = s * NSP + q;
          r_dble[i] = b[i] - tmp[i];
          r[i] = cf((float)r_dble[i].real(), (float)r_dble[i].imag());
        }
      r_sq = norm2_cb(g, r_dble.data(), 1);
      rNorm = std::sqrt(r_sq);
      maxrr = rNorm;
      if (updateX) {
        for (long s : odd)
          for (int q = 0; q < NSP; ++q) {
            const long i = s * NSP + q;
            psi[i] += x_dble[i];
            x[i] = 0;
            b[i] = r_dble[i];
          }
        r0Norm = rNorm;
        maxrx = rNorm;
      }
    }
    if (r_sq < rsd_sq) {
      for (long s : odd)
        for (int q = 0; q < NSP; ++q) psi[s * NSP + q] += cd(x[s * NSP + q]);
      res.n_count = k;  // the loop index at convergence, as the reference reports it (:264)
      break;
    }
  }
  res.resid = true_resid_linop(A, chi, psi);
  res.rel_resid = res.resid / std::sqrt(norm2_cb(g, chi, 1));
  return res;
}

// InvMultiPrecRichardson (lib/actions/ferm/invert/inv_multiprec_richardson.cc:13-107): the FP64
// defect correction r = b - A x; repeat { dx = Dinv r in single precision; x += dx; r -= A dx in
// double } until |r|^2 <= RsdTarget^2 |b|^2, then the true residual.  Dinv here is a plain
// single-precision BiCGStab on A (the InvBiCGStab recursion of invbicgstab.cc:12-200 on float
// fields, inner products summed in double) to relative tolerance inner_tol.  n_count = total inner
// iterations; the outer step count goes to *outer.
static SolveResult richardson_bicgstab(const Op<double>& A, const Op<float>& AF, const cd* chi, cd* psi, double rsd,
                                       double inner_tol, int maxit, int* outer) {
  const Geom& g = *A.g;
  const long N = g.V * NSP;
  const auto& odd = g.sites[1];
  using cf = std::complex<float>;
  std::vector<cd> r(N), tmp(N), dx(N);
  std::vector<cf> rr(N), rr0(N), e(N), p(N), v(N), t(N);
  auto dot = [&](const std::vector<cf>& a, const std::vector<cf>& c) {
    double re = 0, im = 0;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
    for (long i = 0; i < (long)odd.size(); ++i)
      for (int k = 0; k < NSP; ++k) {
        const long q = odd[i] * NSP + k;
        const cd u = std::conj(cd(a[q])) * cd(c[q]);
        re += u.real();
        im += u.imag();
      }
    return cd(re, im);
  };
  SolveResult res{0, 0, 0};
  const double rsd_t = rsd * rsd * norm2_cb(g, chi, 1);
  eo_op(A, tmp.data(), psi, +1);
  for (long s : odd)
    for (int k = 0; k < NSP; ++k) r[s * NSP + k] = chi[s * NSP + k] - tmp[s * NSP + k];
  double rnorm = norm2_cb(g, r.data(), 1);
  int steps = 0;
  while (rnorm > rsd_t && steps < 100 && res.n_count < maxit) {
    ++steps;
    // Dinv: single-precision BiCGStab on A e = r from e = 0
    for (long s : odd)
      for (int k = 0; k < NSP; ++k) {
        const long q = s * NSP + k;
        rr[q] = rr0[q] = cf((float)r[q].real(), (float)r[q].imag());
        e[q] = p[q] = v[q] = 0;
      }
    const double in_sq = inner_tol * inner_tol * dot(rr, rr).real();
    cd rho_prev = 1.0, alpha = 1.0, omega = 1.0;
    for (int k = 1; k <= maxit - res.n_count; ++k) {
      const cd rho = dot(rr0, rr);
      if (rho == cd(0.0)) break;
      const cf beta((rho / rho_prev) * (alpha / omega)), om0(omega);
      for (long s : odd)
        for (int q = 0; q < NSP; ++q) {
          const long i = s * NSP + q;
          p[i] = rr[i] + beta * (p[i] - om0 * v[i]);
        }
      eo_op(AF, v.data(), p.data(), +1);
      alpha = rho / dot(rr0, v);
      rho_prev = rho;
      const cf al(alpha);
      for (long s : odd)
        for (int q = 0; q < NSP; ++q) rr[s * NSP + q] -= al * v[s * NSP + q];
      eo_op(AF, t.data(), rr.data(), +1);
      omega = dot(t, rr) / dot(t, t).real();
      const cf om(omega);
      for (long s : odd)
        for (int q = 0; q < NSP; ++q) {
          const long i = s * NSP + q;
          e[i] += om * rr[i] + al * p[i];
          rr[i] -= om * t[i];
        }
      ++res.n_count;
      if (dot(rr, rr).real() < in_sq) break;
    }
    // x += dx; r -= A dx in double
    for (long s : odd)
      for (int k = 0; k < NSP; ++k) dx[s * NSP + k] = cd(e[s * NSP + k]);
    eo_op(A, tmp.data(), dx.data(), +1);
    for (long s : odd)
      for (int k = 0; k < NSP; ++k) {
        const long q = s * NSP + k;
        psi[q] += dx[q];
        r[q] -= tmp[q];
      }
    rnorm = norm2_cb(g, r.data(), 1);
  }
  if (outer) *outer = steps;
  res.resid = true_resid_linop(A, chi, psi);
  res.rel_resid = res.resid / std::sqrt(norm2_cb(g, chi, 1));
  return res;
}

// FGMRES (NDefl = 0) following lib/actions/ferm/invert/syssolver_linop_fgmres_dr.{h:31-148,
// cc:77-195, 256-273, 459-765}.  The preconditioner is a callback on full-lattice arrays.
// ---------------------------------------------------------------------------------------------
typedef void (*precond_fn)(void* user, cd* out, const cd* in);

struct Givens {
  int col;
  cd s, c, r;
  Givens(int col_, const std::vector<std::vector<cd>>& H) : col(col_) {
    cd f = H[col][col], gg = H[col][col + 1];
    if (f == 0.0) { c = 0; s = 1; r = gg; }
    else if (gg == 0.0) { s = 0; c = std::conj(f) / std::abs(f); r = std::abs(f); }
    else {
      double t = std::sqrt(std::norm(f) + std::norm(gg));
      r = t; c = f / t; s = gg / t;
    }
  }
  void apply_col(int j, std::vector<std::vector<cd>>& H) const {
    if (j == col) { H[col][col] = r; H[col][col + 1] = 0; return; }
    cd a = H[j][col], b = H[j][col + 1];
    H[j][col] = std::conj(c) * a + std::conj(s) * b;
    H[j][col + 1] = -s * a + c * b;
  }
  void apply_vec(std::vector<cd>& v) const {
    cd a = v[col], b = v[col + 1];
    v[col] = std::conj(c) * a + std::conj(s) * b;
    v[col + 1] = -s * a + c * b;
  }
};

// Backward substitution R eta = g on the first n_cols rows of the upper-triangular R
// (LeastSquaresSolve, syssolver_linop_fgmres_dr.cc:256-273); R[col][row] as H.
static void least_squares(const std::vector<std::vector<cd>>& R, const std::vector<cd>& gvec, std::vector<cd>& eta,
                          int n_cols) {
  eta[n_cols - 1] = gvec[n_cols - 1] / R[n_cols - 1][n_cols - 1];
  for (int row = n_cols - 2; row >= 0; --row) {
    eta[row] = gvec[row];
    for (int col = row + 1; col < n_cols; ++col) eta[row] -= R[col][row] * eta[col];
    eta[row] /= R[row][row];
  }
}

// The matrices of one Arnoldi cycle: H[j][i] is column j, row i (Chroma's H(j,i)); R is H with the
// cycle's Givens rotations applied (upper triangular); g the rotated right-hand side |r| e_0.
struct ArnoldiCycle {
  std::vector<std::vector<cd>> H, R;
  std::vector<cd> g;
  std::vector<Givens> rots;
  explicit ArnoldiCycle(int nk) : H(nk, std::vector<cd>(nk + 1, 0.0)), R(H), g(nk + 1, 0.0) {}
};

// One flexible Arnoldi cycle without deflation (FlexibleArnoldiT, syssolver_linop_fgmres_dr.cc:78-195):
// z_j = M v_j, w = A z_j, one modified Gram-Schmidt pass of w against v_0..v_j into column j of H,
// v_{j+1} = w / |w|, column j of R = H's column with the earlier rotations applied, then a new rotation
// that zeroes R(j, j+1), applied to g too.  The cycle ends when |g_{j+1}| <= target (the accumulated
// residual norm), at a happy breakdown (|w| < 1e-14: dimension j), after nkrylov columns or when
// iters reaches maxit.  V[0] and cy.g[0] are set by the caller.  Returns the cycle's dimension.
static int flexible_arnoldi(const Op<double>& A, int nkrylov, double target, int maxit, int& iters,
                            precond_fn prec, void* user, std::vector<std::vector<cd>>& V,
                            std::vector<std::vector<cd>>& Z, std::vector<cd>& w, ArnoldiCycle& cy) {
  const Geom& g = *A.g;
  const auto& odd = g.sites[1];
  auto& H = cy.H;
  auto& R = cy.R;
  int dim = 0;
  for (int j = 0; j < nkrylov && iters < maxit; ++j) {
    if (prec) prec(user, Z[j].data(), V[j].data());
    else for (long s : odd) for (int k = 0; k < NSP; ++k) Z[j][s * NSP + k] = V[j][s * NSP + k];
    eo_op(A, w.data(), Z[j].data(), +1);
    for (int i = 0; i <= j; ++i) {
      H[j][i] = inner_cb(g, V[i].data(), w.data(), 1);
      axpby_cb<double, cd>(g, -H[j][i], V[i].data(), 1.0, w.data(), 1);
    }
    double wnorm = std::sqrt(norm2_cb(g, w.data(), 1));
    H[j][j + 1] = wnorm;
    ++iters;
    if (std::fabs(wnorm) < 1e-14) return j;  // happy breakdown (cc:118-127)
    for (long s : odd) for (int k = 0; k < NSP; ++k) V[j + 1][s * NSP + k] = w[s * NSP + k] / wnorm;
    for (int i = 0; i <= j + 1; ++i) R[j][i] = H[j][i];
    for (int i = 0; i < j; ++i) cy.rots[i].apply_col(j, R);
    cy.rots.emplace_back(j, R);
    cy.rots[j].apply_col(j, R);
    cy.rots[j].apply_vec(cy.g);
    dim = j + 1;
    if (std::fabs(cy.g[j + 1].real()) <= target) break;
  }
  return dim;
}

static SolveResult fgmres(const Op<double>& A, const cd* chi, cd* psi, double rsd_target, int nkrylov, int maxit,
                          precond_fn prec, void* user) {
  const Geom& g = *A.g;
  const long N = g.V * NSP;
  const auto& odd = g.sites[1];
  SolveResult res{0, 0, 0};
  double norm_rhs = std::sqrt(norm2_cb(g, chi, 1));
  double target = norm_rhs * rsd_target;
  std::vector<cd> r(N), tmp(N), w(N);
  std::vector<std::vector<cd>> V(nkrylov + 1, std::vector<cd>(N)), Z(nkrylov, std::vector<cd>(N));
  auto resid = [&]() {
    eo_op(A, tmp.data(), psi, +1);
    for (long s : odd) for (int k = 0; k < NSP; ++k) r[s * NSP + k] = chi[s * NSP + k] - tmp[s * NSP + k];
    return std::sqrt(norm2_cb(g, r.data(), 1));
  };
  double r_norm = resid();
  int iters = 0;
  while (r_norm > target && iters < maxit) {
    ArnoldiCycle cy(nkrylov);
    cy.g[0] = r_norm;
    for (long s : odd) for (int k = 0; k < NSP; ++k) V[0][s * NSP + k] = r[s * NSP + k] / r_norm;
    int dim = flexible_arnoldi(A, nkrylov, target, maxit, iters, prec, user, V, Z, w, cy);
    if (dim == 0) break;
    std::vector<cd> eta(dim);
    least_squares(cy.R, cy.g, eta, dim);
    for (int j = 0; j < dim; ++j) axpby_cb<double, cd>(g, eta[j], Z[j].data(), 1.0, psi, 1);
    r_norm = resid();
  }
  res.n_count = iters;
  res.resid = r_norm;
  res.rel_resid = r_norm / norm_rhs;
  return res;
}

}  // namespace orc

// =============================================================================================
// extern "C" surface used by the Python wrapper (oracle/oracle.py)
// =============================================================================================
using namespace orc;

struct orc_ctx {
  Geom* g;
  Op<double>* op;
  Op<float>* opf;
};

extern "C" {

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

void orc_gamma(double* out) {  // 4 x 4 x 4 complex, then gamma_5 (4 x 4 complex)
  init_gamma();
  cd* o = reinterpret_cast<cd*>(out);
  for (int m = 0; m < 4; ++m)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b) o[(m * 4 + a) * 4 + b] = GAMMA[m][a][b];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) o[64 + a * 4 + b] = GAMMA5[a][b];
}

double orc_uniform(uint64_t seed, uint64_t k) { return runiform(seed, k); }
double orc_normal(uint64_t seed, uint64_t k) { return rnormal(seed, k); }

// Hot-start links: U = reunit(exp(i eps H)), H = (G + G^dag)/2 - tr/3, G_ij = n(2j') + i n(2j'+1)
// with normals numbered k = (s*4 + mu)*18 + 2*(3*row + col) + {0,1}.
void orc_gauge_hot(const int* dims, double eps, uint64_t seed, double* out) {
  Geom g(dims);
  cd* u = reinterpret_cast<cd*>(out);
#pragma omp parallel for schedule(static)
  for (long s = 0; s < g.V; ++s)
    for (int mu = 0; mu < 4; ++mu) {
      M3 G;
      uint64_t base = ((uint64_t)s * 4 + mu) * 18;
      for (int e = 0; e < 9; ++e) G.a[e / 3][e % 3] = cd(rnormal(seed, base + 2 * e), rnormal(seed, base + 2 * e + 1));
      M3 H = mscale(madd(G, madj(G)), 0.5);
      cd tr = mtrace(H) / 3.0;
      for (int i = 0; i < 3; ++i) H.a[i][i] -= tr;
      M3 U = reunit_m3(mexp_taylor(mscale(H, cd(0, eps))));
      store_m3(&u[(s * 4 + mu) * 9], U);
    }
}

void orc_reunit(const int* dims, double* links) {
  Geom g(dims);
  cd* u = reinterpret_cast<cd*>(links);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < g.V * 4; ++i) store_m3(&u[i * 9], reunit_m3(load_m3(&u[i * 9])));
}

// n_smear stout steps of size rho in the directions with smear_dir[mu] != 0 (stout_utils.cc:936-966)
void orc_stout(const int* dims, double* links, double rho, int n_smear, const int* smear_dir) {
  Geom g(dims);
  cd* u = reinterpret_cast<cd*>(links);
  std::vector<cd> cur(u, u + g.V * 36), nxt;
  for (int i = 0; i < n_smear; ++i) { stout_step(g, cur, nxt, rho, smear_dir); cur.swap(nxt); }
  std::copy(cur.begin(), cur.end(), u);
}

// SimpleFermBC::modify (lib/actions/ferm/fermbcs/simple_fermbc.h:87-104) for boundary[m] = bc[m]
void orc_apply_bc(const int* dims, double* links, const int* bc) {
  Geom g(dims);
  cd* u = reinterpret_cast<cd*>(links);
  for (long s = 0; s < g.V; ++s) {
    int x[4];
    g.coords(s, x);
    for (int m = 0; m < 4; ++m)
      if (bc[m] != 1 && x[m] == g.L[m] - 1)
        for (int e = 0; e < 9; ++e) u[(s * 4 + m) * 9 + e] *= (double)bc[m];
  }
}

// Average plaquette Re tr(U_p)/3 over the 6 planes and the link trace Re tr(U)/3.
void orc_plaquette(const int* dims, const double* links, double* plaq, double* link_trace) {
  Geom g(dims);
  std::vector<cd> u(reinterpret_cast<const cd*>(links), reinterpret_cast<const cd*>(links) + g.V * 36);
  double sp = 0, sl = 0;
#pragma omp parallel for reduction(+ : sp, sl) schedule(static)
  for (long s = 0; s < g.V; ++s) {
    for (int mu = 0; mu < 4; ++mu) {
      sl += std::real(mtrace(link(u, s, mu))) / 3.0;
      for (int nu = mu + 1; nu < 4; ++nu) {
        M3 p = mmul(mmul(mmul(link(u, s, mu), link(u, g.fwd[mu][s], nu)), madj(link(u, g.fwd[nu][s], mu))), madj(link(u, s, nu)));
        sp += std::real(mtrace(p)) / 3.0;
      }
    }
  }
  *plaq = sp / (6.0 * g.V);
  *link_trace = sl / (4.0 * g.V);
}

// F(mu,nu) for the 6 planes: out[(s*6 + k)*9 + row*3 + col]
void orc_mesfield(const int* dims, const double* links, double* out) {
  Geom g(dims);
  std::vector<cd> u(reinterpret_cast<const cd*>(links), reinterpret_cast<const cd*>(links) + g.V * 36);
  std::vector<M3> f;
  mesfield(g, u, f);
  cd* o = reinterpret_cast<cd*>(out);
  for (long i = 0; i < 6 * g.V; ++i) store_m3(&o[i * 9], f[i]);
}

// Build the operator from BC-applied links.  link_coeff[mu] multiplies the dslash links
// (makeFermCoeffs, lib/io/aniso_io.cc:63-80); the clover term uses the links as given.
orc_ctx* orc_create(const int* dims, const double* links, double mass, double csw_r, double csw_t, int aniso,
                    double xi_0, double nu, int t_dir, int twisted, double twisted_m) {
  init_gamma();
  orc_ctx* c = new orc_ctx;
  c->g = new Geom(dims);
  const Geom& g = *c->g;
  const cd* u = reinterpret_cast<const cd*>(links);
  std::vector<cd> uin(u, u + g.V * 36);
  CloverParams p{mass, csw_r, csw_t, aniso, xi_0, nu, t_dir};
  c->op = new Op<double>;
  Op<double>& op = *c->op;
  op.g = c->g;
  op.u = uin;
  if (aniso)
    for (long s = 0; s < g.V; ++s)
      for (int m = 0; m < 4; ++m)
        if (m != t_dir)
          for (int e = 0; e < 9; ++e) op.u[(s * 4 + m) * 9 + e] *= nu / xi_0;
  make_clover(g, uin, p, op.clov);
  op.invclov = op.clov;
  double ld = 0;
  int nneg = 0;
  for (long s : g.sites[0]) ldl_invert_site(op.invclov[s], ld, nneg);
  op.logdet_even = ld;
  op.nneg = nneg;
  double ld_odd = 0;
  int nneg_odd = 0;
  for (long s : g.sites[1]) ldl_invert_site(op.invclov[s], ld_odd, nneg_odd);
  op.logdet_odd = ld_odd;
  op.twisted = twisted != 0;
  op.twisted_m = twisted_m;
  // single-precision copy for the reliable CG inner operator
  c->opf = new Op<float>;
  Op<float>& of = *c->opf;
  of.g = c->g;
  of.u.resize(op.u.size());
  for (size_t i = 0; i < op.u.size(); ++i) of.u[i] = std::complex<float>((float)op.u[i].real(), (float)op.u[i].imag());
  auto cvt = [](const std::vector<CloverSite<double>>& a, std::vector<CloverSite<float>>& b) {
    b.resize(a.size());
    for (size_t s = 0; s < a.size(); ++s)
      for (int k = 0; k < 2; ++k) {
        for (int i = 0; i < 6; ++i) b[s].diag[k][i] = (float)a[s].diag[k][i];
        for (int i = 0; i < 15; ++i) b[s].offd[k][i] = std::complex<float>((float)a[s].offd[k][i].real(), (float)a[s].offd[k][i].imag());
      }
  };
  cvt(op.clov, of.clov);
  cvt(op.invclov, of.invclov);
  of.twisted = op.twisted;
  of.twisted_m = (float)twisted_m;
  return c;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  delete c->op;
  delete c->opf;
  delete c->g;
  delete c;
}

long orc_volume(orc_ctx* c) { return c->g->V; }
double orc_logdet_even(orc_ctx* c) { return c->op->logdet_even; }
// sum over the odd sites of log|d| of A's LDL^dag factors (seoprec_clover_linop_w.cc:490-492)
double orc_logdet_odd(orc_ctx* c) { return c->op->logdet_odd; }
int orc_neg_eigs(orc_ctx* c) { return c->op->nneg; }

// Packed clover (72 doubles/site) of A and of A^-1, all sites.
void orc_get_clover(orc_ctx* c, double* clov, double* invclov) {
  std::memcpy(clov, c->op->clov.data(), sizeof(CloverSite<double>) * c->g->V);
  std::memcpy(invclov, c->op->invclov.data(), sizeof(CloverSite<double>) * c->g->V);
}

// Invert packed blocks in place on all sites (used to test the LDL^dag restatement alone)
double orc_clover_invert_packed(long nsites, double* packed) {
  CloverSite<double>* T = reinterpret_cast<CloverSite<double>*>(packed);
  double ld = 0;
  int nn = 0;
  for (long s = 0; s < nsites; ++s) ldl_invert_site(T[s], ld, nn);
  return ld;
}

// op codes shared with the C-ABI: 0 D (hopping term, output parity cb), 1 A (clover, parity cb),
// 2 A^-1 (parity cb), 3 M~ (odd), 4 M~^dag M~ (odd), 5 unpreconditioned M (full),
// 6 symmetric M_s (odd), 7 M_s^dag M_s (odd)
int orc_apply(orc_ctx* c, int opcode, int isign, int cb, double* out, const double* in) {
  cd* o = reinterpret_cast<cd*>(out);
  const cd* i = reinterpret_cast<const cd*>(in);
  const Op<double>& op = *c->op;
  switch (opcode) {
    case 0: dslash(op, o, i, isign, cb); return 0;
    case 1: clover_apply(op, op.clov, o, i, cb); return 0;
    case 2: clover_apply(op, op.invclov, o, i, cb); return 0;
    case 3: eo_op(op, o, i, isign); return 0;
    case 4: {
      std::vector<cd> t(c->g->V * NSP);
      eo_op(op, t.data(), i, +1);
      eo_op(op, o, t.data(), -1);
      return 0;
    }
    case 5: unprec_op(op, o, i, isign); return 0;
    case 6: sym_op(op, o, i, isign); return 0;
    case 7: {
      std::vector<cd> t(c->g->V * NSP);
      sym_op(op, t.data(), i, +1);
      sym_op(op, o, t.data(), -1);
      return 0;
    }
  }
  return -1;
}

// Same operators in single precision (the reliable CG inner operator) on complex64 arrays.
int orc_apply_f32(orc_ctx* c, int opcode, int isign, int cb, float* out, const float* in) {
  auto* o = reinterpret_cast<std::complex<float>*>(out);
  const auto* i = reinterpret_cast<const std::complex<float>*>(in);
  const Op<float>& op = *c->opf;
  switch (opcode) {
    case 0: dslash(op, o, i, isign, cb); return 0;
    case 1: clover_apply(op, op.clov, o, i, cb); return 0;
    case 2: clover_apply(op, op.invclov, o, i, cb); return 0;
    case 3: eo_op(op, o, i, isign); return 0;
    case 6: sym_op(op, o, i, isign); return 0;
  }
  return -1;
}

double orc_norm2_cb(orc_ctx* c, const double* x, int cb) { return norm2_cb(*c->g, reinterpret_cast<const cd*>(x), cb); }

void orc_inner_cb(orc_ctx* c, const double* x, const double* y, int cb, double* out) {
  cd v = inner_cb(*c->g, reinterpret_cast<const cd*>(x), reinterpret_cast<const cd*>(y), cb);
  out[0] = v.real();
  out[1] = v.imag();
}

// solver: 0 = CG (LinOpSysSolverCG), 1 = reliable CG (LinOpSysSolverReliableCGClover), 2 = FGMRES,
// 3 = BiCGStab (LinOpSysSolverBiCGStab, syssolver_linop_bicgstab.h:57-75), 4 = reliable mixed
// BiCGStab (LinOpSysSolverReliableBiCGStabClover, syssolver_linop_rel_bicgstab_clover.h),
// 5 = multi-precision Richardson around a single-precision BiCGStab (inner tolerance = delta);
// res[3] = outer steps (solver 5)
// res[0] = n_count, res[1] = resid, res[2] = rel resid
int orc_solve(orc_ctx* c, int solver, double* psi, const double* chi, double rsd, int maxit, double delta,
              int nkrylov, precond_fn prec, void* user, double* res) {
  cd* x = reinterpret_cast<cd*>(psi);
  const cd* b = reinterpret_cast<const cd*>(chi);
  SolveResult r{0, 0, 0};
  const Geom& g = *c->g;
  if (solver == 0) {
    r = linop_cg(*c->op, b, x, rsd, maxit);
  } else if (solver == 1) {
    // syssolver_linop_rel_cg_clover.h:104-152: chi' = M^dag chi, reliable CG on M^dag M
    std::vector<cd> chit(g.V * NSP);
    eo_op(*c->op, chit.data(), b, -1);
    r = reliable_cg(*c->op, *c->opf, chit.data(), x, rsd, delta, maxit);
    r.resid = true_resid_linop(*c->op, b, x);
    r.rel_resid = r.resid / std::sqrt(norm2_cb(g, b, 1));
  } else if (solver == 2) {
    r = fgmres(*c->op, b, x, rsd, nkrylov, maxit, prec, user);
  } else if (solver == 3) {
    r = invbicgstab(*c->op, b, x, rsd, maxit);
  } else if (solver == 4) {
    r = rel_bicgstab(*c->op, *c->opf, b, x, rsd, delta, maxit);
  } else if (solver == 5) {
    int outer = 0;
    r = richardson_bicgstab(*c->op, *c->opf, b, x, rsd, delta, maxit, &outer);
    res[3] = outer;
  } else {
    return -1;
  }
  res[0] = r.n_count;
  res[1] = r.resid;
  res[2] = r.rel_resid;
  return 0;
}

// Full propagator solve for one source (eoprec_fermact_qprop.cc:41-80 wrapping LinOpSysSolverCG):
// Schur prep on the odd sites, CG solve, even reconstruction, full unpreconditioned residual.
int orc_qprop(orc_ctx* c, double* psi, const double* chi, double rsd, int maxit, double* res) {
  const Geom& g = *c->g;
  const Op<double>& op = *c->op;
  cd* x = reinterpret_cast<cd*>(psi);
  const cd* b = reinterpret_cast<const cd*>(chi);
  const long N = g.V * NSP;
  std::vector<cd> t1(N), t2(N), chit(N), r(N);
  clover_apply(op, op.invclov, t1.data(), b, 0);
  dslash(op, t2.data(), t1.data(), +1, 1);  // oddEvenLinOp = -1/2 D
  for (long s : g.sites[1]) for (int k = 0; k < NSP; ++k) chit[s * NSP + k] = b[s * NSP + k] + 0.5 * t2[s * NSP + k];
  SolveResult sr = linop_cg(op, chit.data(), x, rsd, maxit);
  dslash(op, t1.data(), x, +1, 0);
  for (long s : g.sites[0]) for (int k = 0; k < NSP; ++k) t2[s * NSP + k] = b[s * NSP + k] + 0.5 * t1[s * NSP + k];
  clover_apply(op, op.invclov, x, t2.data(), 0);
  unprec_op(op, r.data(), x, +1);
  double rr = 0, bb = 0;
  for (long i = 0; i < N; ++i) { rr += std::norm(r[i] - b[i]); bb += std::norm(b[i]); }
  res[0] = sr.n_count;
  res[1] = std::sqrt(rr);
  res[2] = std::sqrt(rr / bb);
  return 0;
}

// NERSC archive reader (12-real "4D_SU3_GAUGE_3x3"-free variant: DATATYPE 4D_SU3_GAUGE, IEEE32BIG
// or IEEE64BIG); rows 0,1 stored, row 2 = conj(row0 x row1).  Returns 0 on success and fills dims,
// links (canonical layout) and the header's PLAQUETTE and LINK_TRACE.
int orc_read_nersc(const char* path, int* dims, double* links, long cap_sites, double* hdr_plaq, double* hdr_trace) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return -1;
  std::string line, dtype = "4D_SU3_GAUGE", fp = "IEEE32BIG";
  int d[4] = {0, 0, 0, 0};
  *hdr_plaq = *hdr_trace = 0;
  bool begun = false;
  while (std::getline(in, line)) {
    if (line.find("BEGIN_HEADER") != std::string::npos) { begun = true; continue; }
    if (line.find("END_HEADER") != std::string::npos) break;
    if (!begun) continue;
    auto eq = line.find('=');
    if (eq == std::string::npos) continue;
    auto trim = [](std::string s) {
      size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
      return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    };
    std::string key = trim(line.substr(0, eq)), val = trim(line.substr(eq + 1));
    if (key == "DIMENSION_1") d[0] = std::stoi(val);
    else if (key == "DIMENSION_2") d[1] = std::stoi(val);
    else if (key == "DIMENSION_3") d[2] = std::stoi(val);
    else if (key == "DIMENSION_4") d[3] = std::stoi(val);
    else if (key == "PLAQUETTE") *hdr_plaq = std::stod(val);
    else if (key == "LINK_TRACE") *hdr_trace = std::stod(val);
    else if (key == "DATATYPE") dtype = val;
    else if (key == "FLOATING_POINT") fp = val;
  }
  for (int m = 0; m < 4; ++m) dims[m] = d[m];
  long V = (long)d[0] * d[1] * d[2] * d[3];
  if (V <= 0) return -2;
  if (links == nullptr || cap_sites < V) return 1;  // dims only
  bool dbl = fp.find("64") != std::string::npos;
  bool big = fp.find("BIG") != std::string::npos;
  int nrow = dtype.find("3x3") != std::string::npos ? 3 : 2;
  int wsz = dbl ? 8 : 4;
  std::vector<unsigned char> buf((size_t)V * 4 * nrow * 6 * wsz);
  in.read(reinterpret_cast<char*>(buf.data()), (std::streamsize)buf.size());
  if ((size_t)in.gcount() != buf.size()) return -3;
  auto rd = [&](size_t idx) -> double {
    unsigned char b[8];
    std::memcpy(b, &buf[idx * wsz], wsz);
    if (big) std::reverse(b, b + wsz);
    if (dbl) { double v; std::memcpy(&v, b, 8); return v; }
    float v; std::memcpy(&v, b, 4); return v;
  };
  cd* u = reinterpret_cast<cd*>(links);
  size_t k = 0;
  for (long s = 0; s < V; ++s)
    for (int mu = 0; mu < 4; ++mu) {
      M3 m = mzero();
      for (int r = 0; r < nrow; ++r)
        for (int col = 0; col < 3; ++col) { m.a[r][col] = cd(rd(k), rd(k + 1)); k += 2; }
      if (nrow == 2) {
        m.a[2][0] = std::conj(m.a[0][1] * m.a[1][2] - m.a[0][2] * m.a[1][1]);
        m.a[2][1] = std::conj(m.a[0][2] * m.a[1][0] - m.a[0][0] * m.a[1][2]);
        m.a[2][2] = std::conj(m.a[0][0] * m.a[1][1] - m.a[0][1] * m.a[1][0]);
      }
      store_m3(&u[(s * 4 + mu) * 9], m);
    }
  return 0;
}

// Givens rotation of syssolver_linop_fgmres_dr.h:31-148 built on column col of H (rows col, col + 1),
// applied to each column in cols and then, when vec is not null, to vec (nrows complex): the
// Givens* fixtures of mainprogs/tests/fgmres_dr_tests.cc:251-375.  H holds ncols columns of nrows
// complex numbers (Chroma's H(col, row)).  Returns -1 on an index outside H.
int orc_givens(int ncols, int nrows, double* H, int col, const int* cols, int ncols_apply, double* vec) {
  if (col < 0 || col >= ncols || col + 1 >= nrows) return -1;
  for (int k = 0; k < ncols_apply; ++k)
    if (cols[k] < 0 || cols[k] >= ncols) return -1;
  cd* h = reinterpret_cast<cd*>(H);
  std::vector<std::vector<cd>> M(ncols, std::vector<cd>(nrows));
  for (int j = 0; j < ncols; ++j) for (int i = 0; i < nrows; ++i) M[j][i] = h[(long)j * nrows + i];
  Givens G(col, M);
  for (int k = 0; k < ncols_apply; ++k) G.apply_col(cols[k], M);
  for (int j = 0; j < ncols; ++j) for (int i = 0; i < nrows; ++i) h[(long)j * nrows + i] = M[j][i];
  if (vec) {
    cd* v = reinterpret_cast<cd*>(vec);
    std::vector<cd> t(v, v + nrows);
    G.apply_vec(t);
    std::copy(t.begin(), t.end(), v);
  }
  return 0;
}

// Backward substitution R x = b over the first n_cols rows of the upper-triangular R (ncols columns of
// nrows complex, n_cols <= ncols, n_cols <= nrows): the testLeastSquares fixture of
// fgmres_dr_tests.cc:527-567.  Returns -1 on bad sizes.
int orc_least_squares(int ncols, int nrows, const double* R, const double* b, int n_cols, double* x) {
  if (n_cols < 1 || n_cols > ncols || n_cols > nrows) return -1;
  const cd* r = reinterpret_cast<const cd*>(R);
  std::vector<std::vector<cd>> M(ncols, std::vector<cd>(nrows));
  for (int j = 0; j < ncols; ++j) for (int i = 0; i < nrows; ++i) M[j][i] = r[(long)j * nrows + i];
  std::vector<cd> bv(reinterpret_cast<const cd*>(b), reinterpret_cast<const cd*>(b) + nrows), eta(n_cols);
  least_squares(M, bv, eta, n_cols);
  std::copy(eta.begin(), eta.end(), reinterpret_cast<cd*>(x));
  return 0;
}

// One flexible Arnoldi cycle of the even-odd operator with the identity preconditioner from
// v_0 = chi / |chi|, g = |chi| e_0, stopping at |g_{j+1}| <= rsd_target |chi| (the arnoldi5 and
// arnoldi5GivensRot fixtures, fgmres_dr_tests.cc:162-249, 377-524).  V: nkrylov + 1 full-lattice
// spinors (odd sites written, the rest zero); H, R: nkrylov columns of nkrylov + 1 complex rows;
// g: nkrylov + 1 complex.  Returns the cycle's dimension, -1 on nkrylov < 1.
int orc_arnoldi(orc_ctx* c, int nkrylov, const double* chi, double rsd_target, double* V_out, double* H_out,
                double* R_out, double* g_out) {
  if (nkrylov < 1) return -1;
  const Geom& g = *c->g;
  const long N = g.V * NSP;
  const cd* b = reinterpret_cast<const cd*>(chi);
  double beta = std::sqrt(norm2_cb(g, b, 1));
  std::vector<std::vector<cd>> V(nkrylov + 1, std::vector<cd>(N, 0.0)), Z(nkrylov, std::vector<cd>(N, 0.0));
  std::vector<cd> w(N, 0.0);
  for (long s : g.sites[1]) for (int k = 0; k < NSP; ++k) V[0][s * NSP + k] = b[s * NSP + k] / beta;
  ArnoldiCycle cy(nkrylov);
  cy.g[0] = beta;
  int iters = 0;
  int dim = flexible_arnoldi(*c->op, nkrylov, rsd_target * beta, nkrylov, iters, nullptr, nullptr, V, Z, w, cy);
  cd* vo = reinterpret_cast<cd*>(V_out);
  for (int j = 0; j <= nkrylov; ++j) std::copy(V[j].begin(), V[j].end(), vo + (long)j * N);
  cd* ho = reinterpret_cast<cd*>(H_out);
  cd* ro = reinterpret_cast<cd*>(R_out);
  for (int j = 0; j < nkrylov; ++j)
    for (int i = 0; i <= nkrylov; ++i) {
      ho[(long)j * (nkrylov + 1) + i] = cy.H[j][i];
      ro[(long)j * (nkrylov + 1) + i] = cy.R[j][i];
    }
  std::copy(cy.g.begin(), cy.g.end(), reinterpret_cast<cd*>(g_out));
  return dim;
}

}  // extern "C"
