// compile-only stand-in: the declarations the adapter takes from this header
// (lib/io/enum_io/enum_quarkspintype_io.h:30-35)
#pragma once
#include "../../chromabase.h"

namespace Chroma {
enum QuarkSpinType { QUARK_SPIN_TYPE_FULL, QUARK_SPIN_TYPE_UPPER, QUARK_SPIN_TYPE_LOWER };
}  // namespace Chroma
