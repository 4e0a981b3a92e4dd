// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "chromabase.h"

namespace Chroma {
template <typename T>
class LinearOperator {
 public:
  virtual ~LinearOperator() {}
  virtual void operator()(T& chi, const T& psi, enum PlusMinus isign) const = 0;
  virtual const Subset& subset() const = 0;
};
}  // namespace Chroma
