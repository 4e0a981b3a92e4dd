// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "linearop.h"
#include "handle.h"

namespace Chroma {
template <typename T>
class MdagMLinOp : public LinearOperator<T> {
 public:
  explicit MdagMLinOp(const Handle<LinearOperator<T> >& A);
  void operator()(T& chi, const T& psi, enum PlusMinus isign) const override;
  const Subset& subset() const override;
};
}  // namespace Chroma
