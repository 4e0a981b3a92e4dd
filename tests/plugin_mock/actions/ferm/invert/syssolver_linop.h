// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "../../../linearop.h"
#include "../../../handle.h"
#include "../../../syssolver.h"

namespace Chroma {
template <typename T>
class LinOpSystemSolver : public SystemSolver<T> {};
}  // namespace Chroma
