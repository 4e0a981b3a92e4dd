// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "../../../linearop.h"
#include "../../../handle.h"
#include "../../../syssolver.h"

namespace Chroma {
template <typename T>
class AbsChronologicalPredictor4D {
 public:
  virtual ~AbsChronologicalPredictor4D() {}
  virtual void operator()(T& psi, const LinearOperator<T>& A, const T& chi) = 0;
  virtual void reset() = 0;
  virtual void newVector(const T& psi) = 0;
};

template <typename T>
class MdagMSystemSolver : public SystemSolver<T> {
 public:
  virtual SystemSolverResults_t operator()(T& psi, const T& chi) const = 0;
  virtual SystemSolverResults_t operator()(T& psi, const T& chi, AbsChronologicalPredictor4D<T>& predictor) const = 0;
};
}  // namespace Chroma
