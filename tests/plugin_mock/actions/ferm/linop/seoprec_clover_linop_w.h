// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "../../../linearop.h"

namespace Chroma {
class SymEvenOddPrecCloverLinOp : public LinearOperator<LatticeFermion> {
 public:
  void operator()(LatticeFermion& chi, const LatticeFermion& psi, enum PlusMinus isign) const override;
  const Subset& subset() const override;
};
}  // namespace Chroma
