// compile-only stand-in: the declarations the adapter takes from this header (lib/util/ferm/transf.h)
#pragma once
#include "../../chromabase.h"

namespace Chroma {
void PropToFerm(const LatticePropagator& b, LatticeFermion& a, int color_index, int spin_index);
void FermToProp(const LatticeFermion& a, LatticePropagator& b, int color_index, int spin_index);
}  // namespace Chroma
