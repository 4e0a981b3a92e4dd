// Block-vector BLAS for the flexible GMRES (krylov.cu).
#pragma once
#include "gbc_kernels.h"

namespace gbc {

constexpr int kMaxKrylov = 33;  // NKrylov + 1 basis vectors at most

struct VecList {
  Spinor v[kMaxKrylov];
};

// result layout (in red.result): [i][re/im][rhs] for i < k  (finalized rows 2k x nrhs)
void multi_cdot(const Geom& g, const VecList& vl, int k, const Spinor& w, const Red& red, cudaStream_t s);
// w += sign * sum_{i<k} coef[i * nrhs + r] * V_i   (complex coefficients in device memory)
void multi_caxpy(const Geom& g, const VecList& vl, int k, const double2* coef, const Spinor& w, double sign,
                 cudaStream_t s);
// y = a[r] x  (y is written only)
void blas_cax(const Geom& g, const double2* a, const Spinor& x, const Spinor& y, cudaStream_t s);

}  // namespace gbc
