// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "chromabase.h"

namespace Chroma {
template <typename T, typename P, typename Q>
class FermState {
 public:
  virtual ~FermState() {}
  virtual const Q& getLinks() const = 0;
};
}  // namespace Chroma
