// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "syssolver_linop.h"
#include "../../../state.h"
#include "../../../handle.h"
#include "../../../factory_stand_in.h"

namespace Chroma {
typedef Singleton<SolverFactory<LinOpSystemSolver<LatticeFermion> > > TheLinOpFermSystemSolverFactory;
}  // namespace Chroma
