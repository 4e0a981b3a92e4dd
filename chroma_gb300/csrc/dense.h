// Small dense complex linear algebra on the host, for the deflated restarts of FGMRES-DR: the
// matrices are at most NKrylov + NDefl + 1 <= 33 on a side, one per right-hand side.
// Matrices are column-major: element (row, col) of an ld-row matrix is M[col * ld + row].
#pragma once
#include <complex>
#include <vector>

namespace gbc {
namespace dense {

using cd = std::complex<double>;

// Complex Schur form A = Q T Q^H of an n x n matrix: T (returned in A) upper triangular with the
// eigenvalues on its diagonal, Q unitary.  Householder reduction to Hessenberg form, then the
// shifted QR algorithm (Wilkinson shifts, Givens rotations, deflation of negligible subdiagonal
// entries).  Returns false if some eigenvalue did not converge in 60 n iterations.
bool schur(int n, std::vector<cd>& A, std::vector<cd>& Q);

// Reorders a complex Schur form (T, Q) so that the k diagonal entries of smallest modulus come
// first, by swaps of adjacent diagonal entries (each a Givens similarity); the first k columns of
// Q then span the invariant subspace of those eigenvalues.
void sort_smallest(int n, std::vector<cd>& T, std::vector<cd>& Q, int k);

// Solves A x = b (A^H x = b when adjoint) by LU with partial pivoting; b is overwritten by x.
// Returns false for a singular A.
bool lu_solve(int n, std::vector<cd> A, std::vector<cd>& b, bool adjoint);

// QR of an m x n matrix (m >= n) by Householder reflections: on return A holds the m x n factor
// with orthonormal columns (the first n columns of Q) and R (n x n, upper triangular) is filled.
void qr_thin(int m, int n, std::vector<cd>& A, std::vector<cd>& R);

}  // namespace dense
}  // namespace gbc
