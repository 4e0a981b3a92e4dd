// Small dense complex linear algebra for the deflated FGMRES restart (dense.h).
#include "dense.h"

#include <algorithm>
#include <cmath>

namespace gbc {
namespace dense {

namespace {

inline cd& at(std::vector<cd>& M, int ld, int r, int c) { return M[(size_t)c * ld + r]; }

// the rotation U = [[conj(c), conj(s)], [-s, c]] that maps (a, b) to (r, 0)
void givens(cd a, cd b, cd& c, cd& s) {
  const double r = std::sqrt(std::norm(a) + std::norm(b));
  if (r == 0.0) {
    c = 1.0;
    s = 0.0;
    return;
  }
  c = a / r;
  s = b / r;
}

// T <- U T U^H on rows / columns (k, k+1), Q <- Q U^H;  U as in givens()
void rotate(int n, std::vector<cd>& T, std::vector<cd>& Q, int k, cd c, cd s, int col_lo, int row_hi) {
  for (int j = col_lo; j < n; ++j) {
    const cd x = at(T, n, k, j), y = at(T, n, k + 1, j);
    at(T, n, k, j) = std::conj(c) * x + std::conj(s) * y;
    at(T, n, k + 1, j) = -s * x + c * y;
  }
  for (int i = 0; i <= row_hi; ++i) {
    const cd x = at(T, n, i, k), y = at(T, n, i, k + 1);
    at(T, n, i, k) = x * c + y * s;
    at(T, n, i, k + 1) = -x * std::conj(s) + y * std::conj(c);
  }
  for (int i = 0; i < n; ++i) {
    const cd x = at(Q, n, i, k), y = at(Q, n, i, k + 1);
    at(Q, n, i, k) = x * c + y * s;
    at(Q, n, i, k + 1) = -x * std::conj(s) + y * std::conj(c);
  }
}

}  // namespace

bool schur(int n, std::vector<cd>& A, std::vector<cd>& Q) {
  Q.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) at(Q, n, i, i) = 1.0;
  // Householder reduction to upper Hessenberg form
  std::vector<cd> v(n);
  for (int k = 0; k + 2 < n; ++k) {
    double xn = 0.0;
    for (int i = k + 1; i < n; ++i) xn += std::norm(at(A, n, i, k));
    xn = std::sqrt(xn);
    if (xn == 0.0) continue;
    const cd x0 = at(A, n, k + 1, k);
    const cd alpha = x0 == 0.0 ? cd(-xn) : -xn * x0 / std::abs(x0);
    for (int i = 0; i < n; ++i) v[i] = 0.0;
    for (int i = k + 1; i < n; ++i) v[i] = at(A, n, i, k);
    v[k + 1] -= alpha;
    double vn = 0.0;
    for (int i = k + 1; i < n; ++i) vn += std::norm(v[i]);
    vn = std::sqrt(vn);
    if (vn == 0.0) continue;
    for (int i = k + 1; i < n; ++i) v[i] /= vn;
    // A <- (I - 2 v v^H) A (I - 2 v v^H),  Q <- Q (I - 2 v v^H)
    for (int j = 0; j < n; ++j) {
      cd d = 0.0;
      for (int i = k + 1; i < n; ++i) d += std::conj(v[i]) * at(A, n, i, j);
      for (int i = k + 1; i < n; ++i) at(A, n, i, j) -= 2.0 * v[i] * d;
    }
    for (int i = 0; i < n; ++i) {
      cd d = 0.0, q = 0.0;
      for (int j = k + 1; j < n; ++j) {
        d += at(A, n, i, j) * v[j];
        q += at(Q, n, i, j) * v[j];
      }
      for (int j = k + 1; j < n; ++j) {
        at(A, n, i, j) -= 2.0 * d * std::conj(v[j]);
        at(Q, n, i, j) -= 2.0 * q * std::conj(v[j]);
      }
    }
    for (int i = k + 2; i < n; ++i) at(A, n, i, k) = 0.0;
  }
  // shifted QR iterations on the Hessenberg matrix
  const double eps = 1e-15;
  int hi = n - 1, iter = 0, total = 0;
  std::vector<cd> cs(n), ss(n);
  while (hi > 0) {
    int l = hi;
    while (l > 0) {
      const double sub = std::abs(at(A, n, l, l - 1));
      const double diag = std::abs(at(A, n, l, l)) + std::abs(at(A, n, l - 1, l - 1));
      if (sub <= eps * (diag > 0 ? diag : 1.0)) {
        at(A, n, l, l - 1) = 0.0;
        break;
      }
      --l;
    }
    if (l == hi) {
      --hi;
      iter = 0;
      continue;
    }
    if (++total > 60 * n) return false;
    // Wilkinson shift: the eigenvalue of the trailing 2x2 block nearer its last diagonal entry
    const cd a = at(A, n, hi - 1, hi - 1), b = at(A, n, hi - 1, hi), c = at(A, n, hi, hi - 1),
             d = at(A, n, hi, hi);
    const cd tr = 0.5 * (a + d);
    const cd disc = std::sqrt(0.25 * (a - d) * (a - d) + b * c);
    cd mu = std::abs(tr + disc - d) < std::abs(tr - disc - d) ? tr + disc : tr - disc;
    if (++iter % 11 == 0) mu = d + std::abs(c);  // exceptional shift against cycling
    for (int i = l; i <= hi; ++i) at(A, n, i, i) -= mu;
    for (int k = l; k < hi; ++k) {
      givens(at(A, n, k, k), at(A, n, k + 1, k), cs[k], ss[k]);
      for (int j = k; j < n; ++j) {
        const cd x = at(A, n, k, j), y = at(A, n, k + 1, j);
        at(A, n, k, j) = std::conj(cs[k]) * x + std::conj(ss[k]) * y;
        at(A, n, k + 1, j) = -ss[k] * x + cs[k] * y;
      }
    }
    for (int k = l; k < hi; ++k) {
      const int rmax = std::min(k + 2, hi);
      for (int i = 0; i <= rmax; ++i) {
        const cd x = at(A, n, i, k), y = at(A, n, i, k + 1);
        at(A, n, i, k) = x * cs[k] + y * ss[k];
        at(A, n, i, k + 1) = -x * std::conj(ss[k]) + y * std::conj(cs[k]);
      }
      for (int i = 0; i < n; ++i) {
        const cd x = at(Q, n, i, k), y = at(Q, n, i, k + 1);
        at(Q, n, i, k) = x * cs[k] + y * ss[k];
        at(Q, n, i, k + 1) = -x * std::conj(ss[k]) + y * std::conj(cs[k]);
      }
    }
    for (int i = l; i <= hi; ++i) at(A, n, i, i) += mu;
  }
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) at(A, n, i, j) = 0.0;
  return true;
}

void sort_smallest(int n, std::vector<cd>& T, std::vector<cd>& Q, int k) {
  for (int p = 0; p < k && p < n; ++p) {
    int m = p;
    for (int i = p + 1; i < n; ++i)
      if (std::abs(at(T, n, i, i)) < std::abs(at(T, n, m, m))) m = i;
    // move entry m up to position p by adjacent swaps: the rotation whose first column is the
    // eigenvector (t12, t22 - t11) of the 2x2 block exchanges its diagonal entries
    for (int q = m - 1; q >= p; --q) {
      const cd t11 = at(T, n, q, q), t12 = at(T, n, q, q + 1), t22 = at(T, n, q + 1, q + 1);
      cd c, s;
      givens(t12, t22 - t11, c, s);
      rotate(n, T, Q, q, c, s, q, std::min(q + 1, n - 1));
      at(T, n, q + 1, q) = 0.0;
      at(T, n, q, q) = t22;
      at(T, n, q + 1, q + 1) = t11;
    }
  }
}

bool lu_solve(int n, std::vector<cd> A, std::vector<cd>& b, bool adjoint) {
  if (adjoint) {
    std::vector<cd> T((size_t)n * n);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) at(T, n, i, j) = std::conj(at(A, n, j, i));
    A.swap(T);
  }
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::abs(at(A, n, i, k)) > std::abs(at(A, n, p, k))) p = i;
    if (at(A, n, p, k) == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(at(A, n, k, j), at(A, n, p, j));
      std::swap(b[k], b[p]);
    }
    for (int i = k + 1; i < n; ++i) {
      const cd f = at(A, n, i, k) / at(A, n, k, k);
      for (int j = k; j < n; ++j) at(A, n, i, j) -= f * at(A, n, k, j);
      b[i] -= f * b[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    cd v = b[i];
    for (int j = i + 1; j < n; ++j) v -= at(A, n, i, j) * b[j];
    b[i] = v / at(A, n, i, i);
  }
  return true;
}

void qr_thin(int m, int n, std::vector<cd>& A, std::vector<cd>& R) {
  // modified Gram-Schmidt with one reorthogonalisation pass (m, n <= 33)
  R.assign((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    for (int pass = 0; pass < 2; ++pass)
      for (int q = 0; q < j; ++q) {
        cd d = 0.0;
        for (int i = 0; i < m; ++i) d += std::conj(at(A, m, i, q)) * at(A, m, i, j);
        for (int i = 0; i < m; ++i) at(A, m, i, j) -= d * at(A, m, i, q);
        at(R, n, q, j) += d;
      }
    double nr = 0.0;
    for (int i = 0; i < m; ++i) nr += std::norm(at(A, m, i, j));
    nr = std::sqrt(nr);
    at(R, n, j, j) = nr;
    if (nr > 0.0)
      for (int i = 0; i < m; ++i) at(A, m, i, j) /= nr;
  }
}

}  // namespace dense
}  // namespace gbc
