// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "chromabase.h"

namespace Chroma {
template <typename T>
class Handle {
 public:
  Handle() = default;
  explicit Handle(T* p) : p_(p) {}
  T* operator->() const { return p_; }
  T& operator*() const { return *p_; }
 private:
  T* p_ = nullptr;
};
}  // namespace Chroma
