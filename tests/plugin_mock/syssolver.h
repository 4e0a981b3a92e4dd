// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "chromabase.h"

namespace Chroma {
struct SystemSolverResults_t {
  int n_count = 0;
  Real resid;
};

template <typename T>
class SystemSolver {
 public:
  virtual ~SystemSolver() {}
  virtual SystemSolverResults_t operator()(T& psi, const T& chi) const = 0;
  virtual const Subset& subset() const = 0;
};
}  // namespace Chroma
